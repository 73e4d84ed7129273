// Host side of the batched 2D vorticity ensembles (sc_ens_* in
// include/specns.h): member storage, the seeded initial vorticity, one
// cooperative launch per RK stage, and the CUDA graph of a whole step.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/specns.h"
#include "sc_ens.cuh"

namespace sc {
int set_last_error(int code, const char* msg);   // sc_runtime.cu
}

namespace {

int efail(int code, const char* msg) { return sc::set_last_error(code, msg); }

#define EC(call)                                                             \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) return efail(e_ == cudaErrorMemoryAllocation ? SC_ERR_NOMEM : SC_ERR_CUDA, \
                                        cudaGetErrorString(e_));             \
  } while (0)

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int ilog(int n) { int l = 0; while ((1 << l) < n) ++l; return l; }

}  // namespace

struct sc_ensemble {
  int prec = SC_FP32;
  size_t csize = 8;
  int nm = 0;
  std::vector<int> n;
  std::vector<double> dt, nu8;
  double alpha = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  void* mem = nullptr;          // all member fields
  void* dmem_members = nullptr; // EnsMember<T>[nm] (batched) then [nm] (one at a time)
  void* tw = nullptr;
  unsigned* bar = nullptr;
  int* err = nullptr;
  int items_y = 0, items_x = 0;
  std::vector<int> my_items_y, my_items_x;
  size_t smem = 0;
  int grid = 0;                 // co-resident blocks of the cooperative launch
  std::vector<size_t> field_off;   // per member: offset (elements) of its first field
  std::vector<long long> field;    // per member: elements per field
  std::vector<int> nxp;
  cudaGraphExec_t graph = nullptr;
  // launch shape: the autotuner's choice among the compiled variants
  int variant = 0;
  bool tuned = false;
  std::vector<double> tune_ms;     // per variant: ms per step of the last tuning (< 0: not run)
};

namespace {

int nvariants(const sc_ensemble* e) { return e->prec == SC_FP32 ? sc::kEnsVariantsF32 : sc::kEnsVariantsF64; }
sc::EnsVariant variant(const sc_ensemble* e, int v) {
  return e->prec == SC_FP32 ? sc::ens_variant_f32(v) : sc::ens_variant_f64(v);
}

template <typename T> int launch_stage(sc_ensemble* e, int stage, const sc::EnsMember<T>* members, int nm,
                                       int items_y, int items_x) {
  sc::EnsArgs<T> ea{};
  ea.m = members;
  ea.nm = nm;
  ea.items_y = items_y;
  ea.items_x = items_x;
  ea.stage = stage;
  ea.tw = static_cast<const sc::C2<T>*>(e->tw);
  ea.bar = e->bar;
  ea.err = e->err;
  const int grid = std::max(1, std::min(e->grid, std::max(items_y, items_x)));
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  const sc::EnsVariant v = variant(e, e->variant);
  cfg.blockDim = dim3(v.nt);
  cfg.dynamicSmemBytes = e->smem;
  cfg.stream = e->stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  void* args[] = {&ea};
  EC(cudaLaunchKernelExC(&cfg, v.kernel, args));
  return SC_OK;
}

// Make variant vi the launch shape: shared-memory limit, co-resident grid,
// and the member tables (tile widths and item ranges depend on the shape).
template <typename T> int select_variant(sc_ensemble* e, int vi) {
  using C = sc::C2<T>;
  const sc::EnsVariant v = variant(e, vi);
  if (!v.kernel) return efail(SC_ERR_INVALID, "no such ensemble variant");
  const size_t smem = sizeof(C) * (size_t)v.smem_elems;
  EC(cudaFuncSetAttribute(v.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int dev = 0, nsm = 0, per = 0;
  EC(cudaGetDevice(&dev));
  EC(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  EC(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, v.kernel, v.nt, smem));
  if (per < 1) return efail(SC_ERR_CUDA, "ensemble stage kernel does not fit on an SM");
  e->smem = smem;
  e->grid = nsm * per;
  const int warps = v.nt / 32;
  std::vector<sc::EnsMember<T>> mb(2 * e->nm);
  C* base = static_cast<C*>(e->mem);
  int iy = 0, ix = 0;
  e->my_items_y.resize(e->nm);
  e->my_items_x.resize(e->nm);
  for (int m = 0; m < e->nm; ++m) {
    auto& d = mb[m];
    const int N = e->n[m];
    d.n = N;
    d.logn = ilog(N);
    d.nxh = N / 2 + 1;
    d.nxp = e->nxp[m];
    d.ptile = v.ypts / N > 16 ? 16 : (v.ypts / N < 1 ? 1 : v.ypts / N);
    d.ntx = (d.nxh + d.ptile - 1) / d.ptile;
    d.field = e->field[m];
    C* f = base + e->field_off[m];
    d.w = f;
    d.s = f + d.field;
    d.acc = f + 2 * d.field;
    d.work = f + 3 * d.field;
    d.dt = (T)e->dt[m];
    d.alpha = (T)e->alpha;
    d.nu8 = (T)e->nu8[m];
    d.scale = (T)(1.0 / ((double)N * N));
    d.item_y0 = iy;
    d.item_x0 = ix;
    e->my_items_y[m] = d.ntx;
    e->my_items_x[m] = (N + warps - 1) / warps;
    iy += d.ntx;
    ix += e->my_items_x[m];
    mb[e->nm + m] = d;
    mb[e->nm + m].item_y0 = 0;
    mb[e->nm + m].item_x0 = 0;
  }
  e->items_y = iy;
  e->items_x = ix;
  EC(cudaMemcpyAsync(e->dmem_members, mb.data(), sizeof(sc::EnsMember<T>) * mb.size(), cudaMemcpyHostToDevice,
                     e->stream));
  EC(cudaStreamSynchronize(e->stream));
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  e->variant = vi;
  return SC_OK;
}

template <typename T> int setup(sc_ensemble* e) {
  using C = sc::C2<T>;
  // twiddles
  std::vector<C> t(sc::WarpTw::TOTAL);
  sc::WarpTw::fill(t.data(), [](double a) { return std::cos(a); }, [](double a) { return std::sin(a); });
  EC(cudaMalloc(&e->tw, sizeof(C) * t.size()));
  EC(cudaMemcpy(e->tw, t.data(), sizeof(C) * t.size(), cudaMemcpyHostToDevice));
  // fields: 6 per member (w, s, acc, work x3)
  size_t total = 0;
  e->field_off.resize(e->nm);
  e->field.resize(e->nm);
  e->nxp.resize(e->nm);
  for (int m = 0; m < e->nm; ++m) {
    const int N = e->n[m];
    e->nxp[m] = (N / 2 + 1 + 15) / 16 * 16;
    e->field[m] = (long long)N * e->nxp[m];
    e->field_off[m] = total;
    total += 6 * (size_t)e->field[m];
  }
  EC(cudaMalloc(&e->mem, sizeof(C) * total));
  EC(cudaMemsetAsync(e->mem, 0, sizeof(C) * total, e->stream));
  EC(cudaMalloc(&e->dmem_members, sizeof(sc::EnsMember<T>) * 2 * e->nm));
  EC(cudaMalloc(&e->bar, 2 * sizeof(unsigned)));
  EC(cudaMemset(e->bar, 0, 2 * sizeof(unsigned)));
  EC(cudaMalloc(&e->err, sizeof(int)));
  EC(cudaMemset(e->err, 0, sizeof(int)));
  e->tune_ms.assign(nvariants(e), -1.0);
  // a pinned variant (SPECNS_ENS_VARIANT) skips the autotuner
  int v0 = 0;
  if (const char* pv = std::getenv("SPECNS_ENS_VARIANT")) {
    v0 = std::atoi(pv);
    if (v0 < 0 || v0 >= nvariants(e)) return efail(SC_ERR_INVALID, "SPECNS_ENS_VARIANT out of range");
    e->tuned = true;
  }
  return select_variant<T>(e, v0);
}

template <typename T> int step_batched(sc_ensemble* e);

// Autotuner: time every compiled variant on this ensemble (one warm-up and
// `trial` plain steps each, CUDA events on the ensemble's stream) and keep
// the fastest.  The member states are saved first and restored after every
// trial, so tuning leaves the ensemble where it was.
template <typename T> int tune(sc_ensemble* e, int trial) {
  using C = sc::C2<T>;
  if (trial < 1) trial = 1;
  size_t wbytes = 0;
  for (int m = 0; m < e->nm; ++m) wbytes += sizeof(C) * (size_t)e->field[m];
  void* save = nullptr;
  EC(cudaMalloc(&save, wbytes));
  auto copy_states = [&](bool to_save) -> int {
    size_t off = 0;
    for (int m = 0; m < e->nm; ++m) {
      char* w = static_cast<char*>(e->mem) + sizeof(C) * e->field_off[m];
      char* b = static_cast<char*>(save) + off;
      const size_t nb = sizeof(C) * (size_t)e->field[m];
      EC(cudaMemcpyAsync(to_save ? b : w, to_save ? w : b, nb, cudaMemcpyDeviceToDevice, e->stream));
      off += nb;
    }
    return SC_OK;
  };
  cudaEvent_t a = nullptr, b = nullptr;
  int rc = copy_states(true);
  if (rc == SC_OK && cudaEventCreate(&a) != cudaSuccess) rc = efail(SC_ERR_CUDA, "event creation failed");
  if (rc == SC_OK && cudaEventCreate(&b) != cudaSuccess) rc = efail(SC_ERR_CUDA, "event creation failed");
  int best = e->variant;
  double best_ms = 1e300;
  for (int v = 0; rc == SC_OK && v < nvariants(e); ++v) {
    rc = select_variant<T>(e, v);
    if (rc == SC_OK) rc = step_batched<T>(e);
    if (rc == SC_OK && cudaEventRecord(a, e->stream) != cudaSuccess) rc = efail(SC_ERR_CUDA, "event record failed");
    for (int i = 0; rc == SC_OK && i < trial; ++i) rc = step_batched<T>(e);
    if (rc == SC_OK && cudaEventRecord(b, e->stream) != cudaSuccess) rc = efail(SC_ERR_CUDA, "event record failed");
    float ms = 0.f;
    if (rc == SC_OK && (cudaEventSynchronize(b) != cudaSuccess || cudaEventElapsedTime(&ms, a, b) != cudaSuccess))
      rc = efail(SC_ERR_CUDA, "event timing failed");
    if (rc == SC_OK) rc = copy_states(false);
    if (rc == SC_OK) {
      e->tune_ms[v] = ms / trial;
      if (ms / trial < best_ms) {
        best_ms = ms / trial;
        best = v;
      }
    }
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (rc == SC_OK) rc = select_variant<T>(e, best);
  cudaStreamSynchronize(e->stream);
  cudaFree(save);
  if (rc == SC_OK) e->tuned = true;
  return rc;
}

template <typename T> int step_batched(sc_ensemble* e) {
  auto* mb = static_cast<const sc::EnsMember<T>*>(e->dmem_members);
  for (int st = 1; st <= 4; ++st)
    if (int r = launch_stage<T>(e, st, mb, e->nm, e->items_y, e->items_x)) return r;
  return SC_OK;
}

template <typename T> int steps_one_at_a_time(sc_ensemble* e, int nsteps) {
  auto* mb = static_cast<const sc::EnsMember<T>*>(e->dmem_members) + e->nm;
  for (int m = 0; m < e->nm; ++m)
    for (int i = 0; i < nsteps; ++i)
      for (int st = 1; st <= 4; ++st)
        if (int r = launch_stage<T>(e, st, mb + m, 1, e->my_items_y[m], e->my_items_x[m])) return r;
  return SC_OK;
}

int check_err(sc_ensemble* e) {
  int v = 0;
  EC(cudaMemcpyAsync(&v, e->err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
  EC(cudaStreamSynchronize(e->stream));
  if (v) {
    cudaMemsetAsync(e->err, 0, sizeof(int), e->stream);
    return efail(SC_ERR_TIMEOUT, "a bounded grid barrier gave up");
  }
  return SC_OK;
}

// Numerical Recipes ran1 (initialize.f90:516-548), fresh stream per member.
struct Ran1 {
  int32_t idum, iy = 0, iv[32] = {0};
  explicit Ran1(int32_t s) : idum(s) {}
  static int32_t lcg(int32_t x) {
    const int32_t k = x / 127773;
    x = 16807 * (x - k * 127773) - 2836 * k;
    return x < 0 ? x + 2147483647 : x;
  }
  double next() {
    if (idum <= 0 || iy == 0) {
      int32_t x = -idum;
      if (x < 1) x = 1;
      for (int j = 40; j >= 1; --j) {
        x = lcg(x);
        if (j <= 32) iv[j - 1] = x;
      }
      iy = iv[0];
      idum = x;
    }
    idum = lcg(idum);
    const int j = iy / (1 + (2147483647 - 1) / 32);
    iy = iv[j];
    iv[j] = idum;
    const double r = (1.0 / 2147483647.0) * (double)iy;
    return r < 1.0 - 1.2e-7 ? r : 1.0 - 1.2e-7;
  }
};

}  // namespace

extern "C" {

int sc_ens_create(int precision, int nmembers, const int* n, const double* dt, const double* nu8, double alpha,
                  sc_ensemble** out) {
  if (!out || !n || !dt || !nu8 || nmembers < 1) return efail(SC_ERR_INVALID, "sc_ens_create: bad arguments");
  *out = nullptr;
  if (precision != SC_FP32 && precision != SC_FP64) return efail(SC_ERR_INVALID, "sc_ens_create: bad precision");
  for (int m = 0; m < nmembers; ++m)
    if (!pow2(n[m]) || n[m] < 64 || n[m] > 1024 || !(dt[m] > 0) || !(nu8[m] >= 0))
      return efail(SC_ERR_INVALID, "sc_ens_create: each N must be a power of two in [64, 1024], dt > 0, nu8 >= 0");
  std::unique_ptr<sc_ensemble> e(new sc_ensemble());
  e->prec = precision;
  e->csize = precision == SC_FP32 ? 8 : 16;
  e->nm = nmembers;
  e->n.assign(n, n + nmembers);
  e->dt.assign(dt, dt + nmembers);
  e->nu8.assign(nu8, nu8 + nmembers);
  e->alpha = alpha;
  EC(cudaStreamCreateWithFlags(&e->own, cudaStreamNonBlocking));
  e->stream = e->own;
  int r = precision == SC_FP32 ? setup<float>(e.get()) : setup<double>(e.get());
  if (r != SC_OK) return r;
  EC(cudaStreamSynchronize(e->stream));
  *out = e.release();
  return SC_OK;
}

int sc_ens_destroy(sc_ensemble* e) {
  if (!e) return SC_OK;
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->graph) cudaGraphExecDestroy(e->graph);
  cudaFree(e->mem);
  cudaFree(e->dmem_members);
  cudaFree(e->tw);
  cudaFree(e->bar);
  cudaFree(e->err);
  if (e->own) cudaStreamDestroy(e->own);
  delete e;
  return SC_OK;
}

int sc_ens_set_stream(sc_ensemble* e, void* stream) {
  if (!e) return efail(SC_ERR_INVALID, "null ensemble");
  e->stream = stream ? static_cast<cudaStream_t>(stream) : e->own;
  if (e->graph) {
    cudaGraphExecDestroy(e->graph);
    e->graph = nullptr;
  }
  return SC_OK;
}

int sc_ens_set_member(sc_ensemble* e, int m, const void* w) {
  if (!e || !w || m < 0 || m >= e->nm) return efail(SC_ERR_INVALID, "sc_ens_set_member: bad arguments");
  const size_t row = e->csize * (e->n[m] / 2 + 1);
  char* dst = static_cast<char*>(e->mem) + e->csize * e->field_off[m];
  EC(cudaMemcpy2DAsync(dst, e->csize * e->nxp[m], w, row, row, e->n[m], cudaMemcpyDefault, e->stream));
  EC(cudaStreamSynchronize(e->stream));
  return SC_OK;
}

int sc_ens_get_member(sc_ensemble* e, int m, void* w) {
  if (!e || !w || m < 0 || m >= e->nm) return efail(SC_ERR_INVALID, "sc_ens_get_member: bad arguments");
  const size_t row = e->csize * (e->n[m] / 2 + 1);
  const char* src = static_cast<const char*>(e->mem) + e->csize * e->field_off[m];
  EC(cudaMemcpy2DAsync(w, row, src, e->csize * e->nxp[m], row, e->n[m], cudaMemcpyDefault, e->stream));
  EC(cudaStreamSynchronize(e->stream));
  return SC_OK;
}

int sc_ens_init(sc_ensemble* e, const int* seeds, double kpeak, double energy) {
  if (!e || !seeds || !(kpeak > 0) || !(energy > 0)) return efail(SC_ERR_INVALID, "sc_ens_init: bad arguments");
  const double pi_ref = 3.1415926536;
  for (int m = 0; m < e->nm; ++m) {
    const int N = e->n[m], nxh = N / 2 + 1;
    std::vector<double> re((size_t)N * nxh), im((size_t)N * nxh);
    Ran1 rng(seeds[m]);
    for (int jj = 0; jj < N; ++jj)          // initialize.f90:485-492 draw order
      for (int ii = 0; ii < nxh; ++ii) {
        const double t1 = rng.next();
        const double t2 = 2.0 * pi_ref * rng.next();
        const double a = std::sqrt(-2.0 * std::log(t1));
        re[(size_t)jj * nxh + ii] = a * std::cos(t2) / std::sqrt(2.0);
        im[(size_t)jj * nxh + ii] = a * std::sin(t2) / std::sqrt(2.0);
      }
    // symmetrize2d (symmetrize.f90:8-30), then the 2/3 mask (initialize.f90:494-496)
    for (int ii = 0; ii < nxh; ++ii) { re[(size_t)(N / 2) * nxh + ii] = 0; im[(size_t)(N / 2) * nxh + ii] = 0; }
    for (int jj = 0; jj < N; ++jj) { re[(size_t)jj * nxh + nxh - 1] = 0; im[(size_t)jj * nxh + nxh - 1] = 0; }
    re[0] = im[0] = 0;
    for (int jj = N / 2 + 1; jj < N; ++jj) {
      re[(size_t)jj * nxh] = re[(size_t)(N - jj) * nxh];
      im[(size_t)jj * nxh] = -im[(size_t)(N - jj) * nxh];
    }
    const double kc = 2.0 * (N / 2) / 3.0;
    double en = 0.0;
    for (int jj = 0; jj < N; ++jj)
      for (int ii = 0; ii < nxh; ++ii) {
        const double ky = jj < N / 2 ? jj : jj - N;
        double k2 = (double)ii * ii + ky * ky;
        const size_t idx = (size_t)jj * nxh + ii;
        if (k2 >= kc * kc) { re[idx] = im[idx] = 0; continue; }
        if (k2 == 0) k2 = 1.1754943508222875e-38;   // k2(1,1) = tiny
        // E(k) ~ k exp(-(k/kpeak)^2) <=> |w^| ~ k exp(-(k/kpeak)^2 / 2)
        const double amp = std::sqrt(k2) * std::exp(-0.5 * k2 / (kpeak * kpeak));
        re[idx] *= amp;
        im[idx] *= amp;
        if (!(jj == 0 && ii == 0)) en += (ii == 0 ? 0.5 : 1.0) * (re[idx] * re[idx] + im[idx] * im[idx]) / k2;
      }
    const double f = std::sqrt(energy / en);
    if (e->prec == SC_FP32) {
      std::vector<float2> h((size_t)N * nxh);
      for (size_t i = 0; i < h.size(); ++i) h[i] = make_float2((float)(f * re[i]), (float)(f * im[i]));
      if (int r = sc_ens_set_member(e, m, h.data())) return r;
    } else {
      std::vector<double2> h((size_t)N * nxh);
      for (size_t i = 0; i < h.size(); ++i) h[i] = make_double2(f * re[i], f * im[i]);
      if (int r = sc_ens_set_member(e, m, h.data())) return r;
    }
  }
  return SC_OK;
}

int sc_ens_tune(sc_ensemble* e, int trial_steps, int* chosen) {
  if (!e) return efail(SC_ERR_INVALID, "null ensemble");
  const int r = e->prec == SC_FP32 ? tune<float>(e, trial_steps) : tune<double>(e, trial_steps);
  if (r) return r;
  if (chosen) *chosen = e->variant;
  return check_err(e);
}

int sc_ens_set_variant(sc_ensemble* e, int v) {
  if (!e || v < 0 || v >= nvariants(e)) return efail(SC_ERR_INVALID, "sc_ens_set_variant: bad arguments");
  const int r = e->prec == SC_FP32 ? select_variant<float>(e, v) : select_variant<double>(e, v);
  if (r) return r;
  e->tuned = true;
  return SC_OK;
}

int sc_ens_variant(sc_ensemble* e, int* v, int* count, double* tune_ms, int* shape) {
  if (!e) return efail(SC_ERR_INVALID, "null ensemble");
  if (v) *v = e->variant;
  if (count) *count = nvariants(e);
  if (tune_ms)
    for (int i = 0; i < nvariants(e); ++i) tune_ms[i] = e->tune_ms[i];
  if (shape) {
    const sc::EnsVariant s = variant(e, e->variant);
    shape[0] = s.nt;
    shape[1] = s.minb;
    shape[2] = s.ypts;
    shape[3] = s.rmax;
    shape[4] = s.outline;
  }
  return SC_OK;
}

int sc_ens_rk4_steps(sc_ensemble* e, int nsteps, int mode) {
  if (!e || nsteps < 0 || mode < 0 || mode > 2) return efail(SC_ERR_INVALID, "sc_ens_rk4_steps: bad arguments");
  const bool f32 = e->prec == SC_FP32;
  if (!e->tuned && nsteps > 0) {
    const char* t = std::getenv("SPECNS_ENS_TUNE");
    if (t && t[0] == '0') {
      e->tuned = true;
    } else if (int r = f32 ? tune<float>(e, 3) : tune<double>(e, 3)) {
      return r;
    }
  }
  if (mode == 2) {
    int r = f32 ? steps_one_at_a_time<float>(e, nsteps) : steps_one_at_a_time<double>(e, nsteps);
    if (r) return r;
    return check_err(e);
  }
  if (mode == 0 && !e->graph && nsteps > 0) {
    // capture one step (four stage launches) once and replay it
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      int r = f32 ? step_batched<float>(e) : step_batched<double>(e);
      cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
      if (r == SC_OK && ce == cudaSuccess && g) {
        if (cudaGraphInstantiate(&e->graph, g, 0) != cudaSuccess) e->graph = nullptr;
      }
      if (g) cudaGraphDestroy(g);
    }
    (void)cudaGetLastError();
  }
  for (int i = 0; i < nsteps; ++i) {
    if (mode == 0 && e->graph) {
      EC(cudaGraphLaunch(e->graph, e->stream));
    } else {
      int r = f32 ? step_batched<float>(e) : step_batched<double>(e);
      if (r) return r;
    }
  }
  return check_err(e);
}

int sc_ens_uses_graph(sc_ensemble* e) { return e && e->graph ? 1 : 0; }

}  // extern "C"
