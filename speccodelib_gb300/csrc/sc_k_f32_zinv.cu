// Compiled instances: zinv kernels, float arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_ZINV(float)
