// Compiled instances: ops kernels, double arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_OPS(double)
SC_DEFINE_TILE(double)
