// Compiled instances: discrete-adjoint kernels, double arithmetic.
#include "sc_dispatch.cuh"
#define ADJ_T double
SC_DEFINE_ADJ(double)
