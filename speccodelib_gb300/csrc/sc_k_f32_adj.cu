// Compiled instances: discrete-adjoint kernels, float arithmetic.
#include "sc_dispatch.cuh"
#define ADJ_T float
SC_DEFINE_ADJ(float)
