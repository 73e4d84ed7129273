// TMA-fed strided-axis passes (y and z).
//
// A pencil tile -- P consecutive kx columns by the N points of the pencil --
// is one box of a 4D tensor map (x = kx, y, z, field), so one thread issues
// the whole tile as one or two cp.async.bulk.tensor loads that land in shared
// memory already in the FFT engine's layout sm[n*P + p].  Loads complete on
// an mbarrier; the CTA transforms one buffer while the next tile streams into
// the other, so HBM stays busy while the FFT stages run.
//
//   pencil_tma_kernel : plain y / z pass over nf fields, persistent over
//                       (tile, outer, field) jobs, double-buffered.
//   zinv_tma_kernel   : z-inverse pass of the right-hand side: v^ tile (3
//                       fields) by TMA, the 6 outputs v^, i k x v^ generated
//                       from shared memory, transformed, stored.
//   zfwd_tma_kernel   : z-forward pass of the Lamb vector (3 fields by TMA,
//                       transformed in place) + the spectral update.
#pragma once
#include "sc_passes.cuh"
#include "sc_tma.cuh"

namespace sc {

template <typename T, int LOGN> struct TmaCfg {
  static constexpr int N = 1 << LOGN;
  static constexpr int U = sizeof(T) / 4;   // 8-byte units per complex element
  // tile width: 64-byte rows for long pencils (two buffers fit twice per SM)
  static constexpr int P = sizeof(T) == 4 ? (LOGN <= 8 ? 16 : 8) : (LOGN <= 8 ? 8 : 4);
  static constexpr int NT_RAW = P * N / 8;
  static constexpr int NT = NT_RAW > 512 ? 512 : (NT_RAW < 32 ? 32 : NT_RAW);
  static constexpr int BOX = N < 256 ? N : 256;   // TMA box extent limit
  static constexpr int NBOX = N / BOX;
  using Engine = FFTEngine<T, LOGN, P, P, NT, true>;
  static constexpr size_t TILE_BYTES = sizeof(C2<T>) * N * P;
  // pipeline depth of pencil_tma_kernel: tiles in flight per CTA
  static constexpr int STAGES = TILE_BYTES <= 16384 ? 4 : 3;
  // zinv uses a narrower tile: 3 inputs + 1 work buffer
  static constexpr int PZ = P >= 8 ? P / 2 : P;
  static constexpr int NTZ_RAW = PZ * N / 8;
  static constexpr int NTZ = NTZ_RAW > 512 ? 512 : (NTZ_RAW < 32 ? 32 : NTZ_RAW);
  // work buffer padded one slot per 8 points: conflict-free first-stage scatter
  using EngineZ = FFTEngine<T, LOGN, PZ, PZ, NTZ, true, 3>;
  static constexpr size_t TILEZ_BYTES = sizeof(C2<T>) * N * PZ;
  static constexpr size_t WORKZ_BYTES = sizeof(C2<T>) * EngineZ::SMEM_ELEMS;
};

// L2 prefetch of the update's operands for a z tile (thread 0; `fmap` is the
// whole field slab with tiles P wide and BOX long in z).
template <typename Cfg, typename T>
__device__ __forceinline__ void prefetch_update_tile(const CUtensorMap* fmap, const StageArgs<T>& st, int kx0,
                                                     int iy) {
#pragma unroll
  for (int i = 0; i < 6; ++i)
    if (i < st.pf_n)
      for (int h = 0; h < Cfg::NBOX; ++h) tma_prefetch_4d(fmap, kx0 * Cfg::U, iy, h * Cfg::BOX, st.pf_slot[i]);
}

// Where a pencil lies: element (p, n) of tile (kx0, outer) of field f is
// base + f*field + outer*outer_stride + n*axis_stride + kx0 + p.
template <typename T> struct TmaPass {
  C2<T>* base;            // field 0 of the group
  long long field;        // elements between fields
  long long axis_stride;
  long long outer_stride;
  int axis;               // 1 = y, 2 = z
  int nouter;             // number of outer slabs (nz for y, ny for z)
  int ntx;                // kx tiles
  int nf;                 // fields
  int* err;               // device error word
};

// Issue the loads of one field tile: box (P, BOX, 1) along y or (P, 1, BOX) along z.
template <typename Cfg>
__device__ __forceinline__ void tma_issue_tile(void* dst, const CUtensorMap* map, uint64_t* bar, int axis,
                                               int kx0, int outer, int f, int P, size_t bytes) {
  mbar_arrive_expect_tx(bar, (uint32_t)bytes);
  for (int h = 0; h < Cfg::NBOX; ++h) {
    char* d = static_cast<char*>(dst) + (size_t)h * Cfg::BOX * P * sizeof(C2<float>) * Cfg::U;
    if (axis == 1) tma_load_4d(d, map, bar, kx0 * Cfg::U, h * Cfg::BOX, outer, f);
    else tma_load_4d(d, map, bar, kx0 * Cfg::U, outer, h * Cfg::BOX, f);
  }
}

template <typename T, int LOGN, bool INV>
__global__ void __launch_bounds__(TmaCfg<T, LOGN>::NT, 2)
pencil_tma_kernel(const __grid_constant__ CUtensorMap map, TmaPass<T> tp, Geom g, const C2<T>* __restrict__ tw) {
  using Cfg = TmaCfg<T, LOGN>;
  // stage-0 writes XOR-rotated (conflict-free 64-byte rows) in the forward
  // pass only: measured 4% faster there, 3% slower in the inverse pass
  using E = FFTEngine<T, LOGN, Cfg::P, Cfg::P, Cfg::NT, true, 0, !INV>;
  using C = C2<T>;
  constexpr int P = Cfg::P;
  constexpr int NS = Cfg::STAGES;
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = align128(smdyn);
  __shared__ __align__(8) uint64_t bars[NS];
  const long long total = (long long)tp.ntx * tp.nouter * tp.nf;
  if (launch_failed(tp.err)) return;
  if (threadIdx.x == 0) {
    for (int b = 0; b < NS; ++b) mbar_init(&bars[b], 1);
    fence_mbar_init();
    fence_proxy_async();
  }
  __syncthreads();
  auto buf = [&](int b) { return reinterpret_cast<C*>(smraw + (size_t)b * Cfg::TILE_BYTES); };
  // field slowest: the CTAs in flight work on neighbouring tiles of one
  // field (field fastest, six fields at the same offset, measured 12%
  // slower for the six-field inverse y-pass)
  auto decode = [&](long long job, int& kx0, int& outer, int& f) {
    const long long per = (long long)tp.ntx * tp.nouter;
    f = (int)(job / per);
    const long long t = job % per;
    kx0 = (int)(t % tp.ntx) * P;
    outer = (int)(t / tp.ntx);
  };
  auto issue = [&](long long job, int b) {
    int kx0, outer, f;
    decode(job, kx0, outer, f);
    tma_issue_tile<Cfg>(buf(b), &map, &bars[b], tp.axis, kx0, outer, f, P, Cfg::TILE_BYTES);
  };
  // prologue: the first NS-1 jobs of this CTA in flight
  if (threadIdx.x == 0) {
    for (int k = 0; k < NS - 1; ++k) {
      const long long jk = blockIdx.x + (long long)k * gridDim.x;
      if (jk < total) issue(jk, k);
    }
  }
  long long job = blockIdx.x;
  for (int it = 0; job < total; job += gridDim.x, ++it) {
    const int b = it % NS;
    const long long ahead = job + (long long)(NS - 1) * gridDim.x;
    if (threadIdx.x == 0 && ahead < total) {
      fence_proxy_async();
      issue(ahead, (it + NS - 1) % NS);
    }
    if (!mbar_wait_bounded(&bars[b], (it / NS) & 1, tp.err)) return;
    // the tile's destination before the transform (its address arithmetic
    // then overlaps the FFT; measured 1.41 -> 1.27 ms for the six-field
    // inverse pass at 512^3)
    int kx0, outer, f;
    decode(job, kx0, outer, f);
    const int nvalid = min(P, g.nxh - kx0);
    C* __restrict__ fp = tp.base + f * tp.field + outer * tp.outer_stride + kx0;
    C out[E::JL][E::RL];
    E::template run_smem<INV>(out, buf(b), tw);
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        if (E::out_pos(a, r, p, n) && p < nvalid) fp[n * tp.axis_stride + p] = out[a][r];
      }
  }
}

// z-inverse pass of one right-hand side (DNS): outputs v (3) and w = i k x v (3).
template <typename T, int LOGN>
__global__ void __launch_bounds__(TmaCfg<T, LOGN>::NTZ, 3)
zinv_tma_kernel(const __grid_constant__ CUtensorMap vmap, ZvArgs<T> za, FieldList<T> out, Geom g,
                const C2<T>* __restrict__ tw, int* err) {
  using Cfg = TmaCfg<T, LOGN>;
  using E = typename Cfg::EngineZ;
  using C = C2<T>;
  constexpr int P = Cfg::PZ;
  constexpr int N = Cfg::N;
  constexpr int NT = Cfg::NTZ;
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = align128(smdyn);
  C* in[3];
  for (int c = 0; c < 3; ++c) in[c] = reinterpret_cast<C*>(smraw + c * Cfg::TILEZ_BYTES);
  C* work = reinterpret_cast<C*>(smraw + 3 * Cfg::TILEZ_BYTES);
  __shared__ __align__(8) uint64_t bar;
  __shared__ double red[NT / 32 + 1];
  const int kx0 = blockIdx.x * P;
  const int iy = blockIdx.y;
  const int nvalid = min(P, g.nxh - kx0);
  const long long zstride = (long long)g.ny * g.nxp;
  const long long base = (long long)iy * g.nxp + kx0;
  const T ky = (T)wavenum(iy, g.ny);
  if (launch_failed(err)) return;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    fence_proxy_async();
    mbar_arrive_expect_tx(&bar, (uint32_t)(3 * Cfg::TILEZ_BYTES));
    for (int c = 0; c < 3; ++c)
      for (int h = 0; h < Cfg::NBOX; ++h)
        tma_load_4d(reinterpret_cast<char*>(in[c]) + (size_t)h * Cfg::BOX * P * sizeof(C), &vmap, &bar,
                    kx0 * Cfg::U, iy, h * Cfg::BOX, c);
  }
  __syncthreads();
  if (!mbar_wait_bounded(&bar, 0, err)) return;
  // forcing band energy of the stage input (force.f90:16-22), FP64
  const bool fsum = za.fs.enabled && ((double)kx0 * kx0 + (double)ky * ky < za.fs.fkmax2);
  if (fsum) {
    double q = 0.0;
    const int kyi = wavenum(iy, g.ny), fk_b = k2_lt(za.fs.fkmax2);
    for (int e = threadIdx.x; e < P * N; e += NT) {
      const int p = e % P, n = e / P;
      const int kx = kx0 + p, kz = wavenum(n, g.nz);
      if (p < nvalid && kx * kx + kyi * kyi + kz * kz < fk_b) {
        double s = 0.0;
        for (int c = 0; c < 3; ++c) s += (double)in[c][e].x * in[c][e].x + (double)in[c][e].y * in[c][e].y;
        q += (kx0 + p == 0) ? 0.5 * s : s;
      }
    }
    double sum = block_sum<NT>(q, red);
    if (threadIdx.x == 0) za.fs.partial[(long long)blockIdx.x * g.ny + iy] = sum;
  }
  for (int f = 0; f < 6; ++f) {
    C x[E::J1][E::R1], o[E::JL][E::RL];
#pragma unroll
    for (int a = 0; a < E::J1; ++a)
#pragma unroll
      for (int r = 0; r < E::R1; ++r) {
        int p, n;
        E::in_pos(a, r, p, n);
        const int e = n * P + p;
        const T kx = (T)(kx0 + p), kz = (T)wavenum(n, g.nz);
        x[a][r] = zv_gen<ZV_DNS>(f, in[0][e], in[1][e], in[2][e], kx, ky, kz, true);
      }
    E::template run<true>(x, o, work, tw);
    C* __restrict__ fp = out.f[f] + base;
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        if (E::out_pos(a, r, p, n) && p < nvalid) fp[n * zstride + p] = o[a][r];
      }
  }
}

// z-forward pass of NIN fields (LES: the Lamb vector and tau_ij, NIN = 9)
// + the spectral update: the fields' tiles stream through a three-deep TMA
// ring, each transformed from shared memory into registers and accumulated
// into w (zfwd_accumulate); a buffer is refilled once its transform has read
// it.  fmap: the NIN fields, tiles P wide along z.
template <typename T, int LOGN, int NIN>
__global__ void __launch_bounds__(TmaCfg<T, LOGN>::NT, 1)
zfwd_fields_tma_kernel(const __grid_constant__ CUtensorMap fmap, StageArgs<T> st, Geom g,
                       const C2<T>* __restrict__ tw, int* err) {
  using Cfg = TmaCfg<T, LOGN>;
  using E = typename Cfg::Engine;
  using C = C2<T>;
  constexpr int P = Cfg::P;
  constexpr int NB = 3;
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = align128(smdyn);
  __shared__ __align__(8) uint64_t bars[NB];
  __shared__ double s_coef;
  auto buf = [&](int b) { return reinterpret_cast<C*>(smraw + (size_t)b * Cfg::TILE_BYTES); };
  const int kx0 = blockIdx.x * P;
  const int iy = blockIdx.y;
  const int nvalid = min(P, g.nxh - kx0);
  const long long zstride = (long long)g.ny * g.nxp;
  const long long base = (long long)iy * g.nxp + kx0;
  const T ky = (T)wavenum(iy, g.ny);
  if (launch_failed(err)) return;
  if (threadIdx.x == 0) {
    for (int b = 0; b < NB; ++b) mbar_init(&bars[b], 1);
    fence_mbar_init();
    fence_proxy_async();
    for (int f = 0; f < NB && f < NIN; ++f)
      tma_issue_tile<Cfg>(buf(f), &fmap, &bars[f], 2, kx0, iy, f, P, Cfg::TILE_BYTES);
  }
  __syncthreads();
  C w[E::JL][E::RL][3];
  for (int f = 0; f < NIN; ++f) {
    const int b = f % NB;
    if (!mbar_wait_bounded(&bars[b], (f / NB) & 1, err)) return;
    C o[E::JL][E::RL];
    E::template run_smem<false>(o, buf(b), tw);   // every read of buf(b) precedes its last barrier
    if (threadIdx.x == 0 && f + NB < NIN) {
      fence_proxy_async();
      tma_issue_tile<Cfg>(buf(b), &fmap, &bars[b], 2, kx0, iy, f + NB, P, Cfg::TILE_BYTES);
    }
    zfwd_accumulate<E, T>(w, o, f, kx0, ky, g);
  }
  zfwd_finish<E, T>(w, st, g, kx0, iy, nvalid, base, zstride, s_coef);
}

// z-forward pass of the Lamb vector + the spectral update (DNS).  MODE: the
// update mode as a compile-time constant (-1: st.mode at run time).  With
// MODE == SM_RK4 and vstore, the new state goes back into the tiles and
// leaves by bulk tensor stores through vmap (st.vout, tiles as lmap); the
// kx = 0 points that the fix-up kernel finishes hold zeros until it writes
// them (stage 4 reads no v: the fix-up needs only acc and the side plane).
// Thread count of zfwd_tma_kernel: for 512- and 256-point pencils 16 points
// per thread, which gives its in-place transforms the two-pass form
// (SC_ZFWD_NT8: 8 points per thread, the radix-8 stages).
template <typename T, int LOGN> struct ZfCfg {
  using Cfg = TmaCfg<T, LOGN>;
#ifdef SC_ZFWD_NT8
  static constexpr int NT = Cfg::NT;
#else
  static constexpr int NT = (LOGN == 9 || LOGN == 8) ? Cfg::P * Cfg::N / 16 : Cfg::NT;
#endif
  using Engine = FFTEngine<T, LOGN, Cfg::P, Cfg::P, NT, true>;
};

template <typename T, int LOGN, int MODE>
__global__ void __launch_bounds__(ZfCfg<T, LOGN>::NT, 2)
zfwd_tma_kernel(const __grid_constant__ CUtensorMap lmap, const __grid_constant__ CUtensorMap vmap, int vstore,
                StageArgs<T> st, Geom g, const C2<T>* __restrict__ tw, int* err) {
  using Cfg = TmaCfg<T, LOGN>;
  using E = typename ZfCfg<T, LOGN>::Engine;
  using C = C2<T>;
  constexpr int P = Cfg::P;
  constexpr int N = Cfg::N;
  constexpr int NT = ZfCfg<T, LOGN>::NT;
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = align128(smdyn);
  C* w[3];
  for (int c = 0; c < 3; ++c) w[c] = reinterpret_cast<C*>(smraw + c * Cfg::TILE_BYTES);
  __shared__ __align__(8) uint64_t bars[3];
  __shared__ double s_coef;
  const int kx0 = blockIdx.x * P;
  const int iy = blockIdx.y;
  const int nvalid = min(P, g.nxh - kx0);
  const long long zstride = (long long)g.ny * g.nxp;
  const long long base = (long long)iy * g.nxp + kx0;
  const T ky = (T)wavenum(iy, g.ny);
  if (launch_failed(err)) return;
  if (threadIdx.x == 0) {
    for (int c = 0; c < 3; ++c) mbar_init(&bars[c], 1);
    fence_mbar_init();
    fence_proxy_async();
    for (int c = 0; c < 3; ++c) {
      mbar_arrive_expect_tx(&bars[c], (uint32_t)Cfg::TILE_BYTES);
      for (int h = 0; h < Cfg::NBOX; ++h)
        tma_load_4d(reinterpret_cast<char*>(w[c]) + (size_t)h * Cfg::BOX * P * sizeof(C), &lmap, &bars[c],
                    kx0 * Cfg::U, iy, h * Cfg::BOX, c);
    }
  }
  const bool fblock = st.forced && ((double)kx0 * kx0 + (double)ky * ky < st.fkmax2);
  const int kyi = wavenum(iy, g.ny), fk_b = k2_lt(st.fkmax2), kc_b = k2_lt(st.kcut2);
  // lower edge of the forcing band (0 for force.f90's k2 < fkmax^2)
  const int flo_b = k2_lt(st.fband_lo2);
  if (fblock && threadIdx.x == 0) {
    if (st.fcoef) {
      s_coef = *st.fcoef;
    } else {
      const double kf = forcing_energy(st.kf_partial, st.kf_tiles, st.kf_ptile, g.ny, st.fkmax2);
      s_coef = st.eps / (2.0 * kf);
    }
  }
  __syncthreads();
  for (int c = 0; c < 3; ++c) {
    if (!mbar_wait_bounded(&bars[c], 0, err)) return;
    E::template run_inplace<false>(w[c], tw);
  }
  // Epilogue in batches of EB points per thread: all state loads of a batch
  // are issued before any of them is used.
  constexpr int EB = NT >= 512 ? 2 : 4;
  const bool tstore = MODE == SM_RK4 && vstore;
  for (int e0 = threadIdx.x; e0 < P * N; e0 += NT * EB) {
    C wv[EB][3], vv[EB][3], av[EB][3];
    bool act[EB];
#pragma unroll
    for (int i = 0; i < EB; ++i) {
      const int e = e0 + i * NT;
      const int p = e % P, iz = e / P;
      act[i] = e < P * N && p < nvalid;
      if (!act[i]) continue;
      const long long idx = base + iz * zstride + p;
      load_state<T, MODE>(st, idx, vv[i], av[i]);
#pragma unroll
      for (int c = 0; c < 3; ++c) wv[i][c] = w[c][e];
    }
#pragma unroll
    for (int i = 0; i < EB; ++i) {
      if (!act[i]) continue;
      const int e = e0 + i * NT;
      const int p = e % P, iz = e / P;
      const int ix = kx0 + p;
      const long long idx = base + iz * zstride + p;
      C* wp = wv[i];
      if (fblock) {
        const int kz = wavenum(iz, g.nz);
        const int k2 = ix * ix + kyi * kyi + kz * kz;
        if (k2 < fk_b && k2 >= flo_b) {
          const T ac = (T)s_coef;
#pragma unroll
          for (int c = 0; c < 3; ++c) wp[c] = cadd(wp[c], cscale(st.sin[c][idx], ac));
        }
      }
      if (st.symmetrize) {
        if (ix == 0) {
          const long long s = ((long long)iz * g.ny + iy) * 3;
#pragma unroll
          for (int c = 0; c < 3; ++c) st.side[s + c] = wp[c];
          if (iz > g.nz / 2 || (iz == 0 && iy > g.ny / 2)) {
            if (tstore)
#pragma unroll
              for (int c = 0; c < 3; ++c) w[c][e] = czero<C>();
            continue;
          }
        }
        if (iy == g.ny / 2 || iz == g.nz / 2 || ix == g.nxh - 1 || (ix == 0 && iy == 0 && iz == 0))
          wp[0] = wp[1] = wp[2] = czero<C>();
      }
      if (tstore) {
        C vn[3];
        finish_point_pre<T, MODE>(st, g, idx, ix, iy, iz, kc_b, wp, vv[i], av[i], vn);
#pragma unroll
        for (int c = 0; c < 3; ++c) w[c][e] = vn[c];
      } else {
        finish_point_pre<T, MODE>(st, g, idx, ix, iy, iz, kc_b, wp, vv[i], av[i]);
      }
    }
  }
  if (tstore) {
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int c = 0; c < 3; ++c)
        for (int h = 0; h < Cfg::NBOX; ++h)
          tma_store_4d(&vmap, reinterpret_cast<char*>(w[c]) + (size_t)h * Cfg::BOX * P * sizeof(C), kx0 * Cfg::U,
                       iy, h * Cfg::BOX, c);
      tma_store_commit();
      tma_store_wait_read<0>();
    }
  }
}

}  // namespace sc
