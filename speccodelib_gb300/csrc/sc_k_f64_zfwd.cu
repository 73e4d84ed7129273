// Compiled instances: zfwd kernels, double arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_ZFWD(double)
