// Discrete adjoint of the IF-RK4 step (DNS right-hand side).
//
// Gradients are taken with respect to the real and imaginary parts of every
// stored half-complex entry (g = dJ/dRe v + i dJ/dIm v).  The adjoint of one
// right-hand side R(s) = P Sym(L(s) + F(s)) for an adjoint lam_w is
//   mu = zero P copy^T lam_w                       (projection and the zeroing
//                                                   are self-adjoint; the kx = 0
//                                                   conjugate copies transpose to
//                                                   accumulations into their sources)
//   phi = R2C^T(mu)/N^3 = C2R(D mu)/(2 N^3)       (D = 2 on kx = 0 and kx = nx/2)
//   lam_s = D' R2C(w x phi) + curl D' R2C(phi x u)  (D' = 2 on 0 < kx < nx/2;
//                                                   the curl is self-adjoint)
//         + [band] a mu - (a c/K_f) 2 w s           (forcing, c = sum Re(conj(mu) s))
// computed by zinv (ZV_ADJ: v, w, phi) -> ypass -> xpass (XP_ADJ) -> ypass ->
// zfwd_adj below, whose epilogue applies the transposed Lawson RK4 stage.
#pragma once
#include "sc_passes.cuh"
#include "sc_tma.cuh"

namespace sc {

enum AdjStage { ADJ4 = 4, ADJ3 = 3, ADJ2 = 2, ADJ1 = 1 };

template <typename T> struct AdjArgs {
  int stage;
  const C2<T>* lt[3];   // masked adjoint of v_{n+1}
  C2<T>* lv[3];         // accumulated adjoint of v_n
  C2<T>* lw[3];         // adjoint of the current stage's RHS (read: band; written: next stage)
  C2<T>* lam[3];        // output of stage 1: adjoint of v_n
  const C2<T>* s[3];    // stage input
  const T* ex;
  const T* ey;
  const T* ez;
  T dt;
  int forced;
  double fkmax2, eps;
  const double* kf_partial;
  const double* c_partial;
  int kf_tiles, kf_ptile;
  int mask_rhs;
  double kcut2;
  // stage 1 only: chain = also start the previous step's adjoint (its masked
  // lam into lt_next, dt/6 of it into lw, what a separate init pass would
  // write); write_lam = store lam itself (the last step: the gradient)
  C2<T>* lt_next[3];
  int chain, write_lam;
};

// Add transformed product field f (0-2: w x phi, 3-5: phi x u), in the
// engine's output layout, to the adjoint lam_s: D' t for f < 3, the curl of
// D' t (i k x t) for f >= 3.
template <typename E, typename T>
__device__ __forceinline__ void adj_accum(C2<T> (&l)[E::JL][E::RL][3], const C2<T> (&o)[E::JL][E::RL], int f,
                                          int kx0, T ky, const Geom& g) {
#pragma unroll
  for (int a = 0; a < E::JL; ++a)
#pragma unroll
    for (int r = 0; r < E::RL; ++r) {
      int p, n;
      E::out_pos(a, r, p, n);
      const int ix = kx0 + p;
      const T dp = (ix == 0 || ix == g.nxh - 1) ? T(1) : T(2);
      const C2<T> t = cscale(o[a][r], dp);
      if (f < 3) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
          if (c == f) l[a][r][c] = cadd(l[a][r][c], t);
      } else {
        // curl of (phi x u)^: i k x t
        const T kx = (T)ix, kz = (T)wavenum(n, g.nz);
        switch (f - 3) {
          case 0:
            l[a][r][1] = cadd(l[a][r][1], cmuli(cscale(t, kz)));
            l[a][r][2] = csub(l[a][r][2], cmuli(cscale(t, ky)));
            break;
          case 1:
            l[a][r][0] = csub(l[a][r][0], cmuli(cscale(t, kz)));
            l[a][r][2] = cadd(l[a][r][2], cmuli(cscale(t, kx)));
            break;
          default:
            l[a][r][0] = cadd(l[a][r][0], cmuli(cscale(t, ky)));
            l[a][r][1] = csub(l[a][r][1], cmuli(cscale(t, kx)));
            break;
        }
      }
    }
}

// Forcing adjoint and the transposed Lawson RK4 stage for lam_s held in the
// engine's output layout.  Thread 0 evaluates the band coefficients; the
// caller's barrier makes them visible (fblock is uniform over the block).
// The state arrays are read through restrict-qualified copies, two points
// at a time with every load issued before the first store: the stores to
// lv / lw would otherwise order each point's loads behind the last point's
// stores.
template <typename E, typename T>
__device__ __forceinline__ void adj_epilogue(C2<T> (&l)[E::JL][E::RL][3], const AdjArgs<T>& aa, const Geom& g,
                                             int kx0, int iy, int nvalid, long long base, long long zstride,
                                             bool fblock, double s_a, double s_b) {
  using C = C2<T>;
  constexpr int NP = E::JL * E::RL;
  constexpr int B = 2;
  const C* __restrict__ lt[3] = {aa.lt[0], aa.lt[1], aa.lt[2]};
  C* __restrict__ lv[3] = {aa.lv[0], aa.lv[1], aa.lv[2]};
  C* __restrict__ lw[3] = {aa.lw[0], aa.lw[1], aa.lw[2]};
  C* __restrict__ lam[3] = {aa.lam[0], aa.lam[1], aa.lam[2]};
  const int stage = aa.stage;
  const T dt = aa.dt;
  const int kyi = wavenum(iy, g.ny), fk_b = k2_lt(aa.fkmax2), kc_b = k2_lt(aa.kcut2);
#pragma unroll
  for (int q0 = 0; q0 < NP; q0 += B) {
    long long idx[B];
    bool ok[B];
    int ixs[B], izs[B];
    C ltv[B][3], lvv[B][3];
#pragma unroll
    for (int b = 0; b < B; ++b) {
      const int q = q0 + b;
      int p = 0, n = 0;
      ok[b] = q < NP && E::out_pos(q / E::RL, q % E::RL, p, n) && p < nvalid;
      ixs[b] = kx0 + p;
      izs[b] = n;
      idx[b] = base + n * zstride + p;
      if (!ok[b]) continue;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (stage != ADJ1) ltv[b][c] = lt[c][idx[b]];
        if (stage == ADJ3 || stage == ADJ2 || stage == ADJ1) lvv[b][c] = lv[c][idx[b]];
      }
    }
#pragma unroll
    for (int b = 0; b < B; ++b) {
      if (!ok[b]) continue;
      const int q = q0 + b;
      C* ls = l[q / E::RL][q % E::RL];
      const int ix = ixs[b], iz = izs[b];
      const int kzi = wavenum(iz, g.nz);
      const int k2i = ix * ix + kyi * kyi + kzi * kzi;
      if (fblock) {
        if (k2i < fk_b) {
          C m[3] = {lw[0][idx[b]], lw[1][idx[b]], lw[2][idx[b]]};
          adj_mu<C, T>(m, ix, iy, iz, g, aa.mask_rhs, kc_b);
          const T sa = (T)s_a, sb = (T)(ix == 0 ? 0.5 * s_b : s_b);
#pragma unroll
          for (int c = 0; c < 3; ++c)
            ls[c] = cadd(ls[c], csub(cscale(m[c], sa), cscale(aa.s[c][idx[b]], sb)));
        }
      }
      const T Ef = aa.ex[ix] * aa.ey[iy] * aa.ez[iz];
      switch (stage) {
        case ADJ4:   // lv = E^2 (lt + ls) ; lw = E dt (lt/3 + ls)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            lv[c][idx[b]] = cscale(cadd(ltv[b][c], ls[c]), Ef * Ef);
            lw[c][idx[b]] = cadd(cscale(ltv[b][c], Ef * dt / T(3)), cscale(ls[c], Ef * dt));
          }
          break;
        case ADJ3:   // lv += E ls ; lw = E dt lt/3 + dt/2 ls
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            lv[c][idx[b]] = cadd(lvv[b][c], cscale(ls[c], Ef));
            lw[c][idx[b]] = cadd(cscale(ltv[b][c], Ef * dt / T(3)), cscale(ls[c], T(0.5) * dt));
          }
          break;
        case ADJ2:   // lv += E ls ; lw = E^2 dt lt/6 + E dt/2 ls
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            lv[c][idx[b]] = cadd(lvv[b][c], cscale(ls[c], Ef));
            lw[c][idx[b]] = cadd(cscale(ltv[b][c], Ef * Ef * dt / T(6)), cscale(ls[c], T(0.5) * Ef * dt));
          }
          break;
        default: {   // stage 1: lam = lv + ls
          const bool cut = k2i >= kc_b && k2i > 0;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const C lm = cadd(lvv[b][c], ls[c]);
            if (aa.write_lam) lam[c][idx[b]] = lm;
            if (aa.chain) {
              const C l0 = cut ? czero<C>() : lm;
              aa.lt_next[c][idx[b]] = l0;
              lw[c][idx[b]] = cscale(l0, dt / T(6));
            }
          }
          break;
        }
      }
    }
  }
}

// Band coefficients of the forcing adjoint (thread 0): a = eps / (2 K_f),
// b = 2 a c / K_f.
template <typename T>
__device__ __forceinline__ void adj_band_coef(const AdjArgs<T>& aa, const Geom& g, double& s_a, double& s_b) {
  const double kf = forcing_energy(aa.kf_partial, aa.kf_tiles, aa.kf_ptile, g.ny, aa.fkmax2);
  const double cc = forcing_energy(aa.c_partial, aa.kf_tiles, aa.kf_ptile, g.ny, aa.fkmax2);
  const double a = aa.eps / (2.0 * kf);
  s_a = a;
  s_b = 2.0 * a * cc / kf;
}

template <typename T, int LOGN>
__global__ void __launch_bounds__(PencilCfg<T, LOGN>::NT, PencilCfg<T, LOGN>::MINB_FUSED)
zfwd_adj_kernel(FieldList<T> fin, AdjArgs<T> aa, Geom g, const C2<T>* __restrict__ tw) {
  using Cfg = PencilCfg<T, LOGN>;
  using E = typename Cfg::Engine;
  using C = C2<T>;
  constexpr int P = Cfg::P;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  __shared__ double s_a, s_b;
  const int kx0 = blockIdx.x * P;
  const int iy = blockIdx.y;
  const int nvalid = min(P, g.nxh - kx0);
  const long long zstride = (long long)g.ny * g.nxp;
  const long long base = (long long)iy * g.nxp + kx0;
  const T ky = (T)wavenum(iy, g.ny);

  C l[E::JL][E::RL][3];
#pragma unroll
  for (int a = 0; a < E::JL; ++a)
#pragma unroll
    for (int r = 0; r < E::RL; ++r) l[a][r][0] = l[a][r][1] = l[a][r][2] = czero<C>();
  for (int f = 0; f < 6; ++f) {
    const C* __restrict__ fp = fin.f[f] + base;
    C in[E::J1][E::R1], o[E::JL][E::RL];
#pragma unroll
    for (int a = 0; a < E::J1; ++a)
#pragma unroll
      for (int r = 0; r < E::R1; ++r) {
        int p, n;
        bool ok = E::in_pos(a, r, p, n) && p < nvalid;
        in[a][r] = ok ? fp[n * zstride + p] : czero<C>();
      }
    E::template run<false>(in, o, sm, tw);
    adj_accum<E, T>(l, o, f, kx0, ky, g);
  }
  const bool fblock = aa.forced && ((double)kx0 * kx0 + (double)ky * ky < aa.fkmax2);
  if (fblock) {
    if (threadIdx.x == 0) {
      double a, b;
      adj_band_coef<T>(aa, g, a, b);
      s_a = a;
      s_b = b;
    }
    __syncthreads();
  }
  adj_epilogue<E, T>(l, aa, g, kx0, iy, nvalid, base, zstride, fblock, s_a, s_b);
}

// The same with the six product tiles fetched by TMA, two in flight: field
// f + 2 loads while field f is transformed.  fidx maps the kernel's field
// order (0-2: w x phi, 3-5: phi x u) to the tensor map's field index.
template <typename T, int LOGN> struct AdjTmaCfg {
  using Cfg = TmaCfg<T, LOGN>;
  // tiles half the pass tiles' width where their rows stay 64 bytes or more
  // (128-byte pass rows): two CTAs of half the threads per SM (256^3 FP32
  // adjoint step 8.67 -> 8.59 ms, 128^3 6% faster; SC_ADJ_WIDE: the pass
  // tiles)
#ifndef SC_ADJ_WIDE
  static constexpr bool NARROW = Cfg::P * sizeof(C2<T>) >= 128;
#else
  static constexpr bool NARROW = false;
#endif
  static constexpr int P = NARROW ? Cfg::P / 2 : Cfg::P;
  static constexpr int MINB = NARROW ? 2 : 1;
  static constexpr int N = Cfg::N;
  static constexpr int NT_RAW = P * N / 8;
  static constexpr int NT = NT_RAW > 512 ? 512 : (NT_RAW < 32 ? 32 : NT_RAW);
  using Engine = FFTEngine<T, LOGN, P, P, NT, true>;
  static constexpr size_t TILE_BYTES = sizeof(C2<T>) * N * P;
  static constexpr size_t SMEM = 2 * TILE_BYTES + kSmemAlignPad;
};

template <typename T, int LOGN>
__global__ void __launch_bounds__(AdjTmaCfg<T, LOGN>::NT, AdjTmaCfg<T, LOGN>::MINB)
zfwd_adj_tma_kernel(const __grid_constant__ CUtensorMap pmap, int4 fidx_lo, int2 fidx_hi, AdjArgs<T> aa, Geom g,
                    const C2<T>* __restrict__ tw, int* err) {
  using AC = AdjTmaCfg<T, LOGN>;
  using Cfg = TmaCfg<T, LOGN>;
  using E = typename AC::Engine;
  using C = C2<T>;
  constexpr int P = AC::P;
  extern __shared__ __align__(128) unsigned char smdyn[];
  unsigned char* smraw = align128(smdyn);
  C* buf[2] = {reinterpret_cast<C*>(smraw), reinterpret_cast<C*>(smraw + AC::TILE_BYTES)};
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ double s_a, s_b;
  const int kx0 = blockIdx.x * P;
  const int iy = blockIdx.y;
  const int nvalid = min(P, g.nxh - kx0);
  const long long zstride = (long long)g.ny * g.nxp;
  const long long base = (long long)iy * g.nxp + kx0;
  const T ky = (T)wavenum(iy, g.ny);
  const int fidx[6] = {fidx_lo.x, fidx_lo.y, fidx_lo.z, fidx_lo.w, fidx_hi.x, fidx_hi.y};
  if (launch_failed(err)) return;
  auto issue = [&](int f) {
    mbar_arrive_expect_tx(&bars[f & 1], (uint32_t)AC::TILE_BYTES);
    for (int h = 0; h < Cfg::NBOX; ++h)
      tma_load_4d(reinterpret_cast<char*>(buf[f & 1]) + (size_t)h * Cfg::BOX * P * sizeof(C), &pmap, &bars[f & 1],
                  kx0 * Cfg::U, iy, h * Cfg::BOX, fidx[f]);
  };
  const bool fblock = aa.forced && ((double)kx0 * kx0 + (double)ky * ky < aa.fkmax2);
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    fence_mbar_init();
    fence_proxy_async();
    issue(0);
    issue(1);
    if (fblock) {
      double a, b;
      adj_band_coef<T>(aa, g, a, b);
      s_a = a;
      s_b = b;
    }
  }
  __syncthreads();
  C l[E::JL][E::RL][3];
#pragma unroll
  for (int a = 0; a < E::JL; ++a)
#pragma unroll
    for (int r = 0; r < E::RL; ++r) l[a][r][0] = l[a][r][1] = l[a][r][2] = czero<C>();
  for (int f = 0; f < 6; ++f) {
    if (!mbar_wait_bounded(&bars[f & 1], (f >> 1) & 1, err)) {
      if (threadIdx.x == 0 && f + 1 < 6) mbar_wait_bounded(&bars[(f + 1) & 1], ((f + 1) >> 1) & 1, nullptr);
      return;
    }
    C o[E::JL][E::RL];
    E::template run_smem<false>(o, buf[f & 1], tw);   // ends with a barrier: the buffer is free
    if (threadIdx.x == 0 && f + 2 < 6) {
      fence_proxy_async();
      issue(f + 2);
    }
    adj_accum<E, T>(l, o, f, kx0, ky, g);
  }
  adj_epilogue<E, T>(l, aa, g, kx0, iy, nvalid, base, zstride, fblock, s_a, s_b);
}

// Transpose of symmetrize's kx = 0 conjugate copies, in place on lw:
// lw(src) += conj(lw(tgt)), lw(tgt) = 0.  Sources and targets are disjoint
// and the map is one-to-one, so the points are independent.
template <typename T>
__global__ void adj_copyT_kernel(FieldList<T> lw, Geom g) {
  using C = C2<T>;
  const long long total = (long long)g.ny * g.nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int iy = (int)(t % g.ny), iz = (int)(t / g.ny);
    if (!(iz > g.nz / 2 || (iz == 0 && iy > g.ny / 2))) continue;
    const int sy = (g.ny - iy) % g.ny, sz = (g.nz - iz) % g.nz;
    const long long d = ((long long)iz * g.ny + iy) * g.nxp, s = ((long long)sz * g.ny + sy) * g.nxp;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      lw.f[c][s] = cadd(lw.f[c][s], cconj(lw.f[c][d]));
      lw.f[c][d] = czero<C>();
    }
  }
}

enum AdjOp { AO_INIT = 0, AO_SHELL_GRAD = 1 };

// AO_INIT: lt = mask(lam) (the 2/3 truncation after the step), lw = dt/6 lt.
// AO_SHELL_GRAD: lam = 2 w k^2 v on shells kmin..kmax (gradient of the shell
// enstrophy, w = 1/2 at kx = 0).
template <typename T> struct AdjOpArgs {
  int op;
  const C2<T>* in[3];
  C2<T>* out1[3];
  C2<T>* out2[3];
  T dt;
  double kcut2;
  int kmin, kmax;
};

template <typename T>
__global__ void __launch_bounds__(256) adj_op_kernel(AdjOpArgs<T> ao, Geom g) {
  using C = C2<T>;
  const long long total = (long long)g.ny * g.nz * g.nxh;
  const int kc_b = k2_lt(ao.kcut2);
  for (Walk3 w(blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x, total, g.nxh,
               g.ny);
       w.ok(); w.next()) {
    const int ix = w.ix;
    const long long idx = w.row() * g.nxp + ix;
    const int kyi = wavenum(w.iy, g.ny), kzi = wavenum(w.iz, g.nz);
    const int k2 = ix * ix + kyi * kyi + kzi * kzi;
    if (ao.op == AO_INIT) {
      const bool cut = k2 >= kc_b && k2 > 0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const C l = cut ? czero<C>() : ao.in[c][idx];
        ao.out1[c][idx] = l;
        ao.out2[c][idx] = cscale(l, ao.dt / T(6));
      }
    } else {
      const int ll = shell_index(k2);
      const bool in = ll >= ao.kmin && ll <= ao.kmax;
      const T f = in ? (T)(2.0 * k2 * (ix == 0 ? 0.5 : 1.0)) : T(0);
#pragma unroll
      for (int c = 0; c < 3; ++c) ao.out1[c][idx] = cscale(ao.in[c][idx], f);
    }
  }
}

}  // namespace sc
