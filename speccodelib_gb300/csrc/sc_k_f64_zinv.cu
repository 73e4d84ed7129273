// Compiled instances: zinv kernels, double arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_ZINV(double)
