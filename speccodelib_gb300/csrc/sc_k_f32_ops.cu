// Compiled instances: ops kernels, float arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_OPS(float)
SC_DEFINE_TILE(float)
