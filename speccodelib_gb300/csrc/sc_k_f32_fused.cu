// Compiled instances: zfwd fused with the next zinv, float arithmetic.
#include "sc_dispatch.cuh"
SC_DEFINE_FUSED(float)
