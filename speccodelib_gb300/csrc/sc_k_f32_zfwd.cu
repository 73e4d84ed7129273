// Compiled instances: zfwd kernels, float arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_ZFWD(float)
