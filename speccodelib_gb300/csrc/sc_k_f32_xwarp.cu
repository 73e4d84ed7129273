// Compiled instances: warp-per-row x-pass, float arithmetic (M = 64, 128, 256).
#include "sc_dispatch.cuh"
SC_DEFINE_XWARP(float, SC_XWARP_CASE(float, 6) SC_XWARP_CASE(float, 7) SC_XWARP_CASE(float, 8))
