// Compiled instances: TMA-fed strided passes, double arithmetic.
#include "sc_dispatch.cuh"
#define TMA_T double
SC_DEFINE_TMA(double)
