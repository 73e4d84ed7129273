// Compiled instances: xpass kernels, double arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_XPASS(double)
