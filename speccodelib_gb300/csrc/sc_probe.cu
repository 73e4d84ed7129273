// FP64 FMA throughput of the current GPU: sc_fp64_peak_probe (include/specns.h).
//
// A measurement helper, not part of the solver: it gives the plain-FP64
// step's roofline its compute ceiling.  Each thread runs eight independent
// dependent chains of fma(x, a, b) (two FP64 flops each), so the FMA pipes,
// not latency, set the rate.  The grid is a fixed multiple of the SM count;
// every loop has a fixed trip count, and nothing waits on anything.
#include <cuda_runtime.h>

#include <cstdio>

#include "../../include/specns.h"

namespace sc {
int set_last_error(int code, const char* msg);   // sc_runtime.cu
}

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;
constexpr int kBlocksPerSM = 4;

__global__ void __launch_bounds__(kThreads) dfma_probe_kernel(double* sink, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1.0 + 1e-3 * (threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  // one store per block keeps the chains live
  if (threadIdx.x == 0) sink[blockIdx.x] = s;
}

int fail(const char* what, cudaError_t e) {
  char buf[256];
  std::snprintf(buf, sizeof buf, "sc_fp64_peak_probe: %s: %s", what, cudaGetErrorString(e));
  return sc::set_last_error(SC_ERR_CUDA, buf);
}

}  // namespace

extern "C" int sc_fp64_peak_probe(double* tflops) {
  if (!tflops) return sc::set_last_error(SC_ERR_INVALID, "sc_fp64_peak_probe: null output");
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail("device query", e);
  const int blocks = sms * kBlocksPerSM;
  const int iters = 1 << 14;
  double* sink = nullptr;
  e = cudaMalloc(&sink, sizeof(double) * blocks);
  if (e != cudaSuccess) return fail("cudaMalloc", e);
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float best = 0.0f;
  e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
    cudaEventRecord(e0, s);
    dfma_probe_kernel<<<blocks, kThreads, 0, s>>>(sink, iters, 0.9999999, 1e-9);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms;
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  cudaFree(sink);
  if (e != cudaSuccess) return fail("probe kernel", e);
  const double flops = 2.0 * kChains * (double)iters * kThreads * blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  return SC_OK;
}
