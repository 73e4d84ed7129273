// FP64 diagnostics of a caller-owned spectral velocity field, with no device
// allocation: sc_diagnostics_noalloc (include/specns.h).
//
// Why it exists: some callers cannot call cudaMalloc.  A time-stepping host
// code that reserves its whole device-memory budget at start-up must not
// allocate inside its step loop (an allocation there can fail, or fragment
// the pool, in the middle of a run), and a caller that keeps several
// asynchronous steps in flight cannot afford the device-wide synchronisation
// that cudaMalloc / cudaFree may imply.  Such a caller owns the velocity
// arrays and the output array; the only scratch the reduction needs -- one
// row of block partial sums per thread block -- lives in the file-scope
// device array below instead of in memory allocated per call or per handle.
//
// Limits and sharing:
//  * The scratch array holds kNoAllocPartialMax doubles (4.04 MiB), enough
//    for every grid this library accepts (nx, ny, nz powers of two up to
//    1024: at most 1024 blocks x (5 + nx/2) partials).  Larger requests are
//    rejected with SC_ERR_INVALID before anything is launched.
//  * Every GPU that loads this library holds the array until the process
//    exits.
//  * All calls on a device share the one array.  Nothing in it has to start
//    at zero: each call's blocks overwrite every partial they later read, and
//    the final kernel overwrites every output entry.  Calls whose kernels
//    overlap on the GPU (different streams without ordering between them)
//    race on the array and give wrong results; serialise them.
//  * The first call on a device, with that device current, looks up the
//    array's device address (cudaGetSymbolAddress) and caches it; make that
//    first call before any stream capture begins.  The cached address is the
//    array's place in the device's primary context: a cudaDeviceReset (or
//    other teardown of that context) unloads the module and leaves the
//    address stale, so this entry point is not for use on a device after a
//    reset.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/specns.h"
#include "sc_ops.cuh"

namespace {
constexpr long long kNoAllocPartialMax = 1024LL * (sc::DQ_N + 512);
constexpr int kMaxDevices = 64;
}  // namespace

static __device__ __align__(256) double sc_noalloc_partial[kNoAllocPartialMax];

namespace sc {
int set_last_error(int code, const char* msg);   // sc_runtime.cu
}

namespace {

std::mutex g_mu;
double* g_scratch[kMaxDevices] = {};

int err(int code, const char* fmt, long long a = 0, long long b = 0) {
  char buf[256];
  std::snprintf(buf, sizeof buf, fmt, a, b);
  return sc::set_last_error(code, buf);
}

// Device address of the scratch array on the current device (set-up once
// per device).  In host code the array's name is only a host-side stand-in.
int scratch_on_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return err(SC_ERR_CUDA, "sc_diagnostics_noalloc: cudaGetDevice failed");
  if (dev < 0 || dev >= kMaxDevices) return err(SC_ERR_INVALID, "sc_diagnostics_noalloc: device %lld out of range", dev);
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, sc_noalloc_partial);
    if (e != cudaSuccess || !p)
      return err(SC_ERR_CUDA, "sc_diagnostics_noalloc: cudaGetSymbolAddress failed on device %lld", dev);
    g_scratch[dev] = static_cast<double*>(p);
  }
  *out = g_scratch[dev];
  return SC_OK;
}

bool pow2_in_range(int n) { return n >= 8 && n <= 1024 && (n & (n - 1)) == 0; }

template <typename T>
int run(const void* vx, const void* vy, const void* vz, int nx, int ny, int nz, double* out,
        cudaStream_t s) {
  sc::Geom g{};
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.nxh = nx / 2 + 1;
  g.nxp = g.nxh;   // the caller's arrays have the reference's pitch nx/2+1
  g.field = (long long)nz * ny * g.nxh;
  sc::DiagArgs<T> da{};
  da.v[0] = static_cast<const sc::C2<T>*>(vx);
  da.v[1] = static_cast<const sc::C2<T>*>(vy);
  da.v[2] = static_cast<const sc::C2<T>*>(vz);
  da.physical = 0;
  da.kmax2 = -1.0;
  da.nshell = nx / 2;
  const long long rows = (long long)ny * nz;
  da.rows_per_block = (int)(rows / 1024 > 1 ? rows / 1024 : 1);
  da.nblocks = (int)((rows + da.rows_per_block - 1) / da.rows_per_block);
  const long long need = (long long)da.nblocks * (sc::DQ_N + da.nshell);
  if (need > kNoAllocPartialMax)
    return err(SC_ERR_INVALID, "sc_diagnostics_noalloc: needs %lld doubles of scratch, the static array holds %lld",
               need, kNoAllocPartialMax);
  double* scratch = nullptr;
  int rc = scratch_on_current_device(&scratch);
  if (rc != SC_OK) return rc;
  da.partial = scratch;
  da.out = out;
  sc::diag_partial_kernel<T><<<da.nblocks, 256, sizeof(double) * da.nshell, s>>>(da, g);
  sc::diag_final_kernel<<<1, 256, 0, s>>>(scratch, da.nblocks, sc::DQ_N + da.nshell, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return err(SC_ERR_CUDA, "sc_diagnostics_noalloc: launch failed");
  return SC_OK;
}

}  // namespace

extern "C" int sc_diagnostics_noalloc(int precision, const void* vx, const void* vy, const void* vz,
                                      int nx, int ny, int nz, double* out, void* stream) {
  if (!vx || !vy || !vz || !out) return err(SC_ERR_INVALID, "sc_diagnostics_noalloc: null pointer");
  if (precision != SC_FP32 && precision != SC_FP64)
    return err(SC_ERR_INVALID, "sc_diagnostics_noalloc: precision must be SC_FP32 or SC_FP64");
  if (!pow2_in_range(nx) || !pow2_in_range(ny) || !pow2_in_range(nz))
    return err(SC_ERR_INVALID, "sc_diagnostics_noalloc: nx, ny, nz must be powers of two in [8, 1024]; the static scratch array is sized for that maximum");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  return precision == SC_FP32 ? run<float>(vx, vy, vz, nx, ny, nz, out, s)
                              : run<double>(vx, vy, vz, nx, ny, nz, out, s);
}
