// Compiled instances: plain kernels, double arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_PLAIN(double)
