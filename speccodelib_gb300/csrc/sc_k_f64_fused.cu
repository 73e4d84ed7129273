// Compiled instances: zfwd fused with the next zinv, double arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_FUSED(double)
