// z-inverse pass of the DNS right-hand side from a stage input held in shared
// memory, and the z-forward pass of IF-RK4 stages 1-3 fused with it.
//
// Unfused, stage k ends with zfwd (transform the Lamb vector along z, force,
// symmetrize, project, RK update: write acc and the next stage input s) and
// stage k+1 starts with zinv (read s, transform s and i k x s back along z).
// Both walk the same (kx tile, ky) pencils, so zfwd_zinv does both per tile
// and s never goes through HBM: 6 field passes fewer per right-hand side
// (write s, read s) and one launch fewer.
//
// The exception is the kx = 0 column: symmetrize copies conj(s(-ky, -kz))
// into its targets, values that belong to another tile.  Tiles with kx0 = 0
// therefore store s as the unfused kernel does; after the kx = 0 fix-up a
// one-tile zinv (grid.x = 1) produces their outputs.  Tiles inside the
// forcing band (kx0^2 + ky^2 < fkmax^2) also store s, which the next stage's
// forcing reads.
//
// Five transforms instead of six: kx and ky are constant along a z pencil, so
// w_z = i kx u_y - i ky u_x is formed pointwise from the transformed u; only
// w_x = i (ky s_z - kz s_y) and w_y = i (kz s_x - kx s_z) carry kz and are
// transformed, half a tile (P/2 pencils) at a time through a half-size work
// buffer.  Shared memory per CTA: the three s tiles + the half work tile,
// 112 KB for 32 KB tiles, so two CTAs share an SM.
#pragma once
#include "sc_tma_passes.cuh"
#include "sc_tmem.cuh"

#ifndef ZI_DIV
#define ZI_DIV 16
#endif
#ifndef ZI_MAX
#define ZI_MAX 256
#endif

namespace sc {

template <typename T> struct FusedArgs {
  FieldList<T> out;   // next stage: u (0-2) and w = i k x u (3-5), z-inverse done
  double* kf_next;    // forcing band sums of the next stage input [tile * ny + iy]
  int store_all;      // also store every tile of the next stage input (adjoint)
};

template <typename T, int LOGN> struct ZiCfg {
  using Cfg = TmaCfg<T, LOGN>;
  // tile width: the strided passes' width (halving it, for more CTAs per SM,
  // measured slower: 32-byte row segments)
  static constexpr int P = Cfg::P;
  static constexpr int N = Cfg::N;
  // two points per thread and radix-8 job at most 256 threads (ZI_DIV 16,
  // ZI_MAX 256), or one job per thread up to 512 (ZI_DIV 8, ZI_MAX 512)
  static constexpr int NT_RAW = P * N / ZI_DIV;
  static constexpr int NT = NT_RAW > ZI_MAX ? ZI_MAX : (NT_RAW < 32 ? 32 : NT_RAW);
#ifndef SC_ZI_EB
  static constexpr int EB = NT >= 512 ? 2 : 4;   // epilogue batch
#else
  static constexpr int EB = SC_ZI_EB;
#endif
  using EngF = FFTEngine<T, LOGN, P, P, NT, true, 0, true>;           // whole tile, in place
  using EngH = FFTEngine<T, LOGN, P / 2, P / 2, NT, true, 0, true>;   // half tile
  static constexpr size_t TILE = sizeof(C2<T>) * (size_t)N * P;
  static constexpr size_t SMEM = 3 * TILE + TILE / 2 + kSmemAlignPad;
  static constexpr bool SUPPORTED = P >= 2 && SMEM <= 113 * 1024;
  // CTAs per SM that the shared memory allows (228 KB, 1 KB reserved per CTA)
  static constexpr int MINB_RAW = (int)(233472 / (SMEM + 1024));
  static constexpr int MINB = MINB_RAW > 4 ? 4 : (MINB_RAW < 1 ? 1 : MINB_RAW);
};

// The outputs of the z-inverse that carry kz, transformed half a tile at a
// time: ZV_DNS w_x, w_y; ZV_SMAG also S13, S23, S33.  The others follow
// pointwise from u (kx and ky are constant along a z pencil): w_z, and for
// ZV_SMAG S11, S12, S22.
template <int MODE> struct ZiFields;
template <> struct ZiFields<ZV_DNS> {
  static constexpr int NKZ = 2, NPW = 1;
  __device__ static constexpr int kz_field(int q) { return 3 + q; }
  __device__ static constexpr int pw_field(int) { return 5; }
};
template <> struct ZiFields<ZV_SMAG> {
  static constexpr int NKZ = 5, NPW = 4;
  __device__ static constexpr int kz_field(int q) { return q < 2 ? 3 + q : (q == 2 ? 8 : (q == 3 ? 10 : 11)); }
  __device__ static constexpr int pw_field(int q) { return q == 0 ? 5 : (q == 1 ? 6 : (q == 2 ? 7 : 9)); }
};
// pointwise output f (5: w_z, 6: S11, 7: S12, 9: S22) from u at (kx, ky)
template <typename C, typename R> __device__ __forceinline__ C zi_pointwise(int f, C ux, C uy, R kx, R ky) {
  switch (f) {
    case 5: return cmuli(csub(cscale(uy, kx), cscale(ux, ky)));
    case 6: return cmuli(cscale(ux, kx));
    case 7: return cmuli(cscale(cadd(cscale(uy, kx), cscale(ux, ky)), R(0.5)));
    default: return cmuli(cscale(uy, ky));
  }
}

// Steps after the stage input s of tile (kx0, iy) is in the three tiles rt
// (natural order, element (p, n) at n*P + p): transform the outputs that
// carry kz (half tiles through `work`), then s in place, and store u and the
// pointwise outputs.  Starts with the tiles complete (caller's barrier);
// ends with a barrier.
// umap: a map of out.f[0..5] tiled as rt (u, and for ZV_DNS w_z, leave the
// tiles by bulk tensor stores), or nullptr (element stores).
template <typename T, int LOGN, int MODE = ZV_DNS>
__device__ __forceinline__ void zinv_from_tiles(C2<T>* const rt[3], C2<T>* work, int kx0, int iy, int nvalid,
                                                long long base, long long zstride, const FieldList<T>& out,
                                                const Geom& g, const C2<T>* __restrict__ tw,
                                                const CUtensorMap* umap) {
  using Z = ZiCfg<T, LOGN>;
  using EH = typename Z::EngH;
  using EF = typename Z::EngF;
  using C = C2<T>;
  constexpr int P = Z::P;
  constexpr int N = Z::N;
  constexpr int NT = Z::NT;
  constexpr int PH = P / 2;
  using ZF = ZiFields<MODE>;
  const T ky = (T)wavenum(iy, g.ny);
#ifndef SC_NO_TMEM_W
  // FP32 512- and 256-point pencils with bulk stores: w_x and w_y as whole-tile
  // two-pass transforms.  Each thread forms its 16 step-1 points of both
  // from the stage-input tiles and parks the step-1 values in TMEM; s
  // becomes u in place; u_z leaves, w_z = i kx u_y - i ky u_x takes its
  // tile, u_x and u_y leave; their tiles are then the exchange buffers that
  // finish w_x and w_y, which leave by bulk stores as well.  No half tiles,
  // no work buffer, no element stores (SC_NO_TMEM_W: the half-tile path).
  if constexpr (MODE == ZV_DNS && EF::TWO_PASS && sizeof(T) == 4) {
    if (umap) {
      using Cfg = TmaCfg<T, LOGN>;
      __shared__ uint32_t s_tmem;
      const int t = threadIdx.x, warp = t >> 5;
      const int p = t % P, j = t / P;
      if (warp == 0) tmem_alloc(&s_tmem, 128);
      tmem_fence_before_sync();
      __syncthreads();
      tmem_fence_after_sync();
      // lanes 32 (warp % 4) .., columns 64 (warp / 4) .. + 63: w_x at +0, w_y at +32
      const uint32_t tw_addr = s_tmem + ((uint32_t)(32 * (warp & 3)) << 16) + 64u * (uint32_t)(warp >> 2);
      const T kx = (T)(kx0 + p);
#pragma unroll 1
      for (int q = 0; q < 2; ++q) {
        C v[16];
#pragma unroll
        for (int m = 0; m < 16; ++m) {
          const int n = j + EF::S1 * m, e = n * P + p;
          v[m] = zv_gen<MODE>(3 + q, rt[0][e], rt[1][e], rt[2][e], kx, ky, (T)wavenum(n, g.nz), true);
        }
        EF::template phase1_512<true>(v, tw);
        uint32_t r[32];
#pragma unroll
        for (int m = 0; m < 16; ++m) {
          r[2 * m] = __float_as_uint(v[m].x);
          r[2 * m + 1] = __float_as_uint(v[m].y);
        }
        tmem_store32(tw_addr + 32u * q, r);
      }
      tmem_wait_store();
      __syncthreads();
      for (int c = 0; c < 3; ++c) EF::template run_inplace<true>(rt[c], tw);
      auto store = [&](int c, int f) {
        for (int h = 0; h < Cfg::NBOX; ++h)
          tma_store_4d(umap, rt[c] + (size_t)h * Cfg::BOX * P, kx0 * Cfg::U, iy, h * Cfg::BOX, f);
      };
      fence_proxy_async();
      __syncthreads();
      if (t == 0) {
        store(2, 2);
        tma_store_commit();
        store(0, 0);
        store(1, 1);
        tma_store_commit();
        tma_store_wait_read<1>();
      }
      __syncthreads();
      for (int e = t; e < P * N; e += NT) {
        const int pe = e % P;
        const C ux = rt[0][e], uy = rt[1][e];
        rt[2][e] = cmuli(csub(cscale(uy, (T)(kx0 + pe)), cscale(ux, ky)));
      }
      fence_proxy_async();
      __syncthreads();
      if (t == 0) {
        store(2, 5);
        tma_store_commit();
        tma_store_wait_read<1>();   // u_x and u_y have left their tiles
      }
      __syncthreads();
#pragma unroll 1
      for (int q = 0; q < 2; ++q) {
        uint32_t r[32];
        tmem_load32(tw_addr + 32u * q, r);
        C v[16];
#pragma unroll
        for (int m = 0; m < 16; ++m) v[m] = mk<C>(__uint_as_float(r[2 * m]), __uint_as_float(r[2 * m + 1]));
        EF::template finish_512<true>(v, rt[q], tw);
      }
      fence_proxy_async();
      tmem_fence_before_sync();
      __syncthreads();
      tmem_fence_after_sync();
      if (t == 0) {
        store(0, 3);
        store(1, 4);
        tma_store_commit();
        tma_store_wait_read<0>();
      }
      if (warp == 0) {
        __syncwarp();   // the warp-collective release after thread 0's stores
        tmem_dealloc(s_tmem, 128);
      }
      __syncthreads();
      return;
    }
  }
#endif
#pragma unroll 1
  for (int q = 0; q < ZF::NKZ; ++q) {
    const int f = ZF::kz_field(q);
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      C x[EH::J1][EH::R1], o[EH::JL][EH::RL];
#pragma unroll
      for (int a = 0; a < EH::J1; ++a)
#pragma unroll
        for (int r = 0; r < EH::R1; ++r) {
          int p, n;
          const bool ok = EH::in_pos(a, r, p, n);
          const int e = ok ? n * P + h * PH + p : 0;   // padding jobs (tiny N) read nothing
          const T kx = (T)(kx0 + h * PH + p), kz = (T)wavenum(n, g.nz);
          x[a][r] = ok ? zv_gen<MODE>(f, rt[0][e], rt[1][e], rt[2][e], kx, ky, kz, true) : czero<C>();
        }
      EH::template run<true>(x, o, work, tw);
      C* __restrict__ fp = out.f[f] + base + h * PH;
#pragma unroll
      for (int a = 0; a < EH::JL; ++a)
#pragma unroll
        for (int r = 0; r < EH::RL; ++r) {
          int p, n;
          if (EH::out_pos(a, r, p, n) && h * PH + p < nvalid) fp[n * zstride + p] = o[a][r];
        }
    }
  }
  for (int c = 0; c < 3; ++c) EF::template run_inplace<true>(rt[c], tw);
#ifdef SC_NO_USTORE
  umap = nullptr;
#endif
  if (umap && MODE != ZV_DNS) {
    // u by bulk stores; the pointwise outputs from the tiles while they drain
    using Cfg = TmaCfg<T, LOGN>;
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int c = 0; c < 3; ++c)
        for (int h = 0; h < Cfg::NBOX; ++h)
          tma_store_4d(umap, rt[c] + (size_t)h * Cfg::BOX * P, kx0 * Cfg::U, iy, h * Cfg::BOX, c);
      tma_store_commit();
    }
    for (int e = threadIdx.x; e < P * N; e += NT) {
      const int p = e % P, n = e / P;
      if (p >= nvalid) continue;
      const C ux = rt[0][e], uy = rt[1][e];
      const T kx = (T)(kx0 + p);
      const long long idx = base + n * zstride + p;
#pragma unroll
      for (int q = 0; q < ZF::NPW; ++q) out.f[ZF::pw_field(q)][idx] = zi_pointwise(ZF::pw_field(q), ux, uy, kx, ky);
    }
    if (threadIdx.x == 0) tma_store_wait_read<0>();
    __syncthreads();
    return;
  }
  if (umap) {
    using Cfg = TmaCfg<T, LOGN>;
    auto store = [&](int c, int f) {
      for (int h = 0; h < Cfg::NBOX; ++h)
        tma_store_4d(umap, rt[c] + (size_t)h * Cfg::BOX * P, kx0 * Cfg::U, iy, h * Cfg::BOX, f);
    };
    fence_proxy_async();
    __syncthreads();
    // u_z first, in a group of its own: its tile takes w_z once read out
    if (threadIdx.x == 0) {
      store(2, 2);
      tma_store_commit();
      store(0, 0);
      store(1, 1);
      tma_store_commit();
      tma_store_wait_read<1>();
    }
    __syncthreads();
    // w_z = i kx u_y - i ky u_x into the u_z tile (u_x, u_y read while they drain)
    for (int e = threadIdx.x; e < P * N; e += NT) {
      const int p = e % P;
      const C ux = rt[0][e], uy = rt[1][e];
      const T kx = (T)(kx0 + p);
      rt[2][e] = cmuli(csub(cscale(uy, kx), cscale(ux, ky)));
    }
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      store(2, 5);
      tma_store_commit();
      tma_store_wait_read<0>();
    }
    __syncthreads();
    return;
  }
  // u and the pointwise outputs, 64-byte row segments
  for (int e = threadIdx.x; e < P * N; e += NT) {
    const int p = e % P, n = e / P;
    if (p >= nvalid) continue;
    const C ux = rt[0][e], uy = rt[1][e], uz = rt[2][e];
    const long long idx = base + n * zstride + p;
    out.f[0][idx] = ux;
    out.f[1][idx] = uy;
    out.f[2][idx] = uz;
    const T kx = (T)(kx0 + p);
#pragma unroll
    for (int q = 0; q < ZF::NPW; ++q) out.f[ZF::pw_field(q)][idx] = zi_pointwise(ZF::pw_field(q), ux, uy, kx, ky);
  }
  __syncthreads();
}

// Standalone z-inverse (MODE ZV_DNS, or ZV_SMAG for the LES operands): the
// stage input tile by TMA, K_f partial sums, then zinv_from_tiles.
// grid = (kx tiles or za.tiles_x, ny).
template <typename T, int LOGN, int MODE>
__global__ void __launch_bounds__(ZiCfg<T, LOGN>::NT, ZiCfg<T, LOGN>::MINB)
zinv5_tma_kernel(const __grid_constant__ CUtensorMap vmap, const __grid_constant__ CUtensorMap umap, ZvArgs<T> za,
                 FieldList<T> out, Geom g, const C2<T>* __restrict__ tw, int* err) {
  using Z = ZiCfg<T, LOGN>;
  using Cfg = TmaCfg<T, LOGN>;
  using C = C2<T>;
  constexpr int P = Z::P;
  constexpr int N = Z::N;
  constexpr int NT = Z::NT;
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = align128(smdyn);
  C* rt[3];
  for (int c = 0; c < 3; ++c) rt[c] = reinterpret_cast<C*>(smraw + c * Z::TILE);
  C* work = reinterpret_cast<C*>(smraw + 3 * Z::TILE);
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
    mbar_arrive_expect_tx(&bar, (uint32_t)(3 * Z::TILE));
    for (int c = 0; c < 3; ++c)
      for (int h = 0; h < Cfg::NBOX; ++h)
        tma_load_4d(reinterpret_cast<char*>(rt[c]) + (size_t)h * Cfg::BOX * P * sizeof(C), &vmap, &bar,
                    kx0 * Cfg::U, iy, h * Cfg::BOX, c);
  }
  __syncthreads();
  if (!mbar_wait_bounded(&bar, 0, err)) return;
  // forcing band energy of the stage input (force.f90:16-22), FP64
  if (za.fs.enabled && ((double)kx0 * kx0 + (double)ky * ky < za.fs.fkmax2)) {
    double q = 0.0;
    const int kyi = wavenum(iy, g.ny), fk_b = k2_lt(za.fs.fkmax2);
    for (int e = threadIdx.x; e < P * N; e += NT) {
      const int p = e % P, n = e / P;
      const int kx = kx0 + p, kz = wavenum(n, g.nz);
      if (p < nvalid && kx * kx + kyi * kyi + kz * kz < fk_b) {
        double s = 0.0;
        for (int c = 0; c < 3; ++c) s += (double)rt[c][e].x * rt[c][e].x + (double)rt[c][e].y * rt[c][e].y;
        q += (kx0 + p == 0) ? 0.5 * s : s;
      }
    }
    const double sum = block_sum<NT>(q, red);
    if (threadIdx.x == 0) za.fs.partial[(long long)blockIdx.x * g.ny + iy] = sum;
  }
  zinv_from_tiles<T, LOGN, MODE>(rt, work, kx0, iy, nvalid, base, zstride, out, g, tw, za.ustore ? &umap : nullptr);
}

// Third operand of the adjoint right-hand side along z:
// phi^ = D (zero P lam) / (2 N^3) (D = 2 on the kx = 0 and kx = nx/2 planes,
// the weights of C2R^T), with the forcing-adjoint band sums
// c = sum Re(conj(mu) v) of the stage input v.  lam tiles by TMA, mu formed
// in shared memory, three in-place transforms.  grid = (kx tiles, ny).
template <typename T, int LOGN>
__global__ void __launch_bounds__(ZiCfg<T, LOGN>::NT, ZiCfg<T, LOGN>::MINB)
zinv_phi_tma_kernel(const __grid_constant__ CUtensorMap lmap, const __grid_constant__ CUtensorMap omap, ZvArgs<T> za,
                    FieldList<T> out, Geom g, const C2<T>* __restrict__ tw, int* err) {
  using Z = ZiCfg<T, LOGN>;
  using Cfg = TmaCfg<T, LOGN>;
  using EF = typename Z::EngF;
  using C = C2<T>;
  constexpr int P = Z::P;
  constexpr int N = Z::N;
  constexpr int NT = Z::NT;
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = align128(smdyn);
  C* rt[3];
  for (int c = 0; c < 3; ++c) rt[c] = reinterpret_cast<C*>(smraw + c * Z::TILE);
  __shared__ __align__(8) uint64_t bar;
  __shared__ double red[NT / 32 + 1];
  const int kx0 = blockIdx.x * P;
  const int iy = blockIdx.y;
  const int nvalid = min(P, g.nxh - kx0);
  const long long zstride = (long long)g.ny * g.nxp;
  const long long base = (long long)iy * g.nxp + kx0;
  const double ky = wavenum(iy, g.ny);
  if (launch_failed(err)) return;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    fence_proxy_async();
    mbar_arrive_expect_tx(&bar, (uint32_t)(3 * Z::TILE));
    for (int c = 0; c < 3; ++c)
      for (int h = 0; h < Cfg::NBOX; ++h)
        tma_load_4d(reinterpret_cast<char*>(rt[c]) + (size_t)h * Cfg::BOX * P * sizeof(C), &lmap, &bar,
                    kx0 * Cfg::U, iy, h * Cfg::BOX, c);
  }
  __syncthreads();
  if (!mbar_wait_bounded(&bar, 0, err)) return;
  const bool fsum = za.fs.enabled && ((double)kx0 * kx0 + ky * ky < za.fs.fkmax2);
  const int kyi = wavenum(iy, g.ny), fk_b = k2_lt(za.fs.fkmax2), kc_b = k2_lt(za.kcut2);
  double q = 0.0;
  for (int e = threadIdx.x; e < P * N; e += NT) {
    const int p = e % P, n = e / P;
    if (p >= nvalid) continue;   // columns beyond nx/2: zeros, never stored
    const int ix = kx0 + p;
    C m[3] = {rt[0][e], rt[1][e], rt[2][e]};
    adj_mu<C, T>(m, ix, iy, n, g, za.mask_rhs, kc_b);
    if (fsum) {
      const int kz = wavenum(n, g.nz);
      if (ix * ix + kyi * kyi + kz * kz < fk_b)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const C sv = za.v[c][base + n * zstride + p];
          q += (double)m[c].x * sv.x + (double)m[c].y * sv.y;
        }
    }
    const T d = (T)((ix == 0 || ix == g.nxh - 1) ? za.inv_n3 : 0.5 * za.inv_n3);
#pragma unroll
    for (int c = 0; c < 3; ++c) rt[c][e] = cscale(m[c], d);
  }
  __syncthreads();
  if (fsum) {
    const double s2 = block_sum<NT>(q, red);
    if (threadIdx.x == 0) za.cpartial[(long long)blockIdx.x * g.ny + iy] = s2;
  }
  // 256- and 512-point pencils (two-pass in-place transforms): phi in place
  // in the tiles, then out by bulk tensor stores (omap tiles the three
  // outputs as lmap tiles lam; columns past nx/2+1 lie outside it and are
  // not written).  Shorter pencils: element stores from the transform's
  // registers (the bulk form gained nothing at 128^3).
  if (EF::TWO_PASS && za.ustore) {
    for (int c = 0; c < 3; ++c) EF::template run_inplace<true>(rt[c], tw);
    fence_proxy_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int c = 0; c < 3; ++c)
        for (int h = 0; h < Cfg::NBOX; ++h)
          tma_store_4d(&omap, reinterpret_cast<char*>(rt[c]) + (size_t)h * Cfg::BOX * P * sizeof(C), kx0 * Cfg::U,
                       iy, h * Cfg::BOX, c);
      tma_store_commit();
      tma_store_wait_read<0>();
    }
    return;
  }
  for (int c = 0; c < 3; ++c) {
    C o[EF::JL][EF::RL];
    EF::template run_smem<true>(o, rt[c], tw);
    C* __restrict__ fp = out.f[c] + base;
#pragma unroll
    for (int a = 0; a < EF::JL; ++a)
#pragma unroll
      for (int r = 0; r < EF::RL; ++r) {
        int p, n;
        if (EF::out_pos(a, r, p, n) && p < nvalid) fp[n * zstride + p] = o[a][r];
      }
  }
}

// z-forward pass of RK stages 1-3 fused with the next stage's z-inverse,
// MODE the stage's update mode (SM_RK1..3; -1: st.mode at run time).
// grid = (kx tiles, ny).
template <typename T, int LOGN, int MODE>
__global__ void __launch_bounds__(ZiCfg<T, LOGN>::NT, ZiCfg<T, LOGN>::MINB)
zfwd_zinv_tma_kernel(const __grid_constant__ CUtensorMap lmap, const __grid_constant__ CUtensorMap fmap,
                     StageArgs<T> st, FusedArgs<T> fa, Geom g, const C2<T>* __restrict__ tw, int* err) {
  using Z = ZiCfg<T, LOGN>;
  using Cfg = TmaCfg<T, LOGN>;
  using EF = typename Z::EngF;
  using C = C2<T>;
  constexpr int P = Z::P;
  constexpr int N = Z::N;
  constexpr int NT = Z::NT;
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = align128(smdyn);
  C* rt[3];
  for (int c = 0; c < 3; ++c) rt[c] = reinterpret_cast<C*>(smraw + c * Z::TILE);
  C* work = reinterpret_cast<C*>(smraw + 3 * Z::TILE);
  __shared__ __align__(8) uint64_t bars[3];
  __shared__ double s_coef;
  __shared__ double red[NT / 32 + 1];
  const int kx0 = blockIdx.x * P;
  const int iy = blockIdx.y;
  const int nvalid = min(P, g.nxh - kx0);
  const long long zstride = (long long)g.ny * g.nxp;
  const long long base = (long long)iy * g.nxp + kx0;
  const T ky = (T)wavenum(iy, g.ny);
  const bool tile0 = kx0 == 0;
  const bool band = st.forced && ((double)kx0 * kx0 + (double)ky * ky < st.fkmax2);
  const int kyi = wavenum(iy, g.ny), fk_b = k2_lt(st.fkmax2), kc_b = k2_lt(st.kcut2);
  if (launch_failed(err)) return;
  if (threadIdx.x == 0) {
    for (int c = 0; c < 3; ++c) mbar_init(&bars[c], 1);
    fence_mbar_init();
    fence_proxy_async();
    for (int c = 0; c < 3; ++c) {
      mbar_arrive_expect_tx(&bars[c], (uint32_t)Z::TILE);
      for (int h = 0; h < Cfg::NBOX; ++h)
        tma_load_4d(reinterpret_cast<char*>(rt[c]) + (size_t)h * Cfg::BOX * P * sizeof(C), &lmap, &bars[c],
                    kx0 * Cfg::U, iy, h * Cfg::BOX, c);
    }
    if (band) {
      const double kf = forcing_energy(st.kf_partial, st.kf_tiles, st.kf_ptile, g.ny, st.fkmax2);
      s_coef = st.eps / (2.0 * kf);
    }
  }
  __syncthreads();
  for (int c = 0; c < 3; ++c) {
    if (!mbar_wait_bounded(&bars[c], 0, err)) return;
    // the update's operands into L2 once the Lamb tiles are in (issued with
    // them, the prefetch delays them)
    if (c == 2 && threadIdx.x == 0) prefetch_update_tile<Cfg>(&fmap, st, kx0, iy);
    EF::template run_inplace<false>(rt[c], tw);
  }
  // spectral update; the next stage input goes back into the tiles
  double q = 0.0;
  constexpr int EB = Z::EB;
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
      for (int c = 0; c < 3; ++c) wv[i][c] = rt[c][e];
    }
#pragma unroll
    for (int i = 0; i < EB; ++i) {
      if (!act[i]) continue;
      const int e = e0 + i * NT;
      const int p = e % P, iz = e / P;
      const int ix = kx0 + p;
      const long long idx = base + iz * zstride + p;
      C* wp = wv[i];
      const int kz = wavenum(iz, g.nz);
      const int k2 = ix * ix + kyi * kyi + kz * kz;
      if (band && k2 < fk_b) {
        const T ac = (T)s_coef;
#pragma unroll
        for (int c = 0; c < 3; ++c) wp[c] = cadd(wp[c], cscale(st.sin[c][idx], ac));
      }
      if (ix == 0) {
        const long long sd = ((long long)iz * g.ny + iy) * 3;
#pragma unroll
        for (int c = 0; c < 3; ++c) st.side[sd + c] = wp[c];
        if (iz > g.nz / 2 || (iz == 0 && iy > g.ny / 2)) continue;
      }
      if (iy == g.ny / 2 || iz == g.nz / 2 || ix == g.nxh - 1 || (ix == 0 && iy == 0 && iz == 0))
        wp[0] = wp[1] = wp[2] = czero<C>();
      C sn[3];
      finish_point_pre<T, MODE>(st, g, idx, ix, iy, iz, kc_b, wp, vv[i], av[i], sn);
      if (tile0 || band || fa.store_all) {
#pragma unroll
        for (int c = 0; c < 3; ++c) st.sout[c][idx] = sn[c];
      }
      if (!tile0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) rt[c][e] = sn[c];
        if (band && k2 < fk_b) {
#pragma unroll
          for (int c = 0; c < 3; ++c) q += (double)sn[c].x * sn[c].x + (double)sn[c].y * sn[c].y;
        }
      }
    }
  }
  if (tile0) return;
  __syncthreads();
  // forcing band energy of the next stage input (force.f90:16-22), FP64
  if (band && fa.kf_next) {
    const double sum = block_sum<NT>(q, red);
    if (threadIdx.x == 0) fa.kf_next[(long long)blockIdx.x * g.ny + iy] = sum;
  }
  // fa.out[0..2] are the Lamb fields: lmap tiles them as rt
  zinv_from_tiles<T, LOGN>(rt, work, kx0, iy, nvalid, base, zstride, fa.out, g, tw, &lmap);
}

}  // namespace sc
