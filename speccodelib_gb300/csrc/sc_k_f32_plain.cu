// Compiled instances: plain kernels, float arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_PLAIN(float)
