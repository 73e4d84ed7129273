// Compiled instances: xpass kernels, float arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_XPASS(float)
