// Compiled instances: TMA-fed strided passes, float arithmetic.
#include "sc_dispatch.cuh"
#define TMA_T float
SC_DEFINE_TMA(float)
