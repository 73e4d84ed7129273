// Compiled instances: warp-per-row x-pass, double arithmetic (M = 64, 128).
#include "sc_dispatch.cuh"
SC_DEFINE_XWARP(double, SC_XWARP_CASE(double, 6) SC_XWARP_CASE(double, 7))
