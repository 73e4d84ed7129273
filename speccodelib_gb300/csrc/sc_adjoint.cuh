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
};

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
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        E::out_pos(a, r, p, n);
        const int ix = kx0 + p;
        const T dp = (ix == 0 || ix == g.nxh - 1) ? T(1) : T(2);
        const C t = cscale(o[a][r], dp);
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
  const bool fblock = aa.forced && ((double)kx0 * kx0 + (double)ky * ky < aa.fkmax2);
  if (fblock) {
    if (threadIdx.x == 0) {
      const double kf = forcing_energy(aa.kf_partial, aa.kf_tiles, aa.kf_ptile, g.ny, aa.fkmax2);
      const double cc = forcing_energy(aa.c_partial, aa.kf_tiles, aa.kf_ptile, g.ny, aa.fkmax2);
      const double a = aa.eps / (2.0 * kf);
      s_a = a;
      s_b = 2.0 * a * cc / kf;
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < E::JL; ++a)
#pragma unroll
    for (int r = 0; r < E::RL; ++r) {
      int p, n;
      if (!(E::out_pos(a, r, p, n) && p < nvalid)) continue;
      const int ix = kx0 + p, iz = n;
      const long long idx = base + n * zstride + p;
      C* ls = l[a][r];
      if (fblock) {
        const double kz = wavenum(iz, g.nz);
        if ((double)ix * ix + (double)ky * ky + kz * kz < aa.fkmax2) {
          C m[3] = {aa.lw[0][idx], aa.lw[1][idx], aa.lw[2][idx]};
          adj_mu<C, T>(m, ix, iy, iz, g, aa.mask_rhs, aa.kcut2);
          const T sa = (T)s_a, sb = (T)(ix == 0 ? 0.5 * s_b : s_b);
#pragma unroll
          for (int c = 0; c < 3; ++c)
            ls[c] = cadd(ls[c], csub(cscale(m[c], sa), cscale(aa.s[c][idx], sb)));
        }
      }
      const T Ef = aa.ex[ix] * aa.ey[iy] * aa.ez[iz];
      const T dt = aa.dt;
      switch (aa.stage) {
        case ADJ4:   // lv = E^2 (lt + ls) ; lw = E dt (lt/3 + ls)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const C lt = aa.lt[c][idx];
            aa.lv[c][idx] = cscale(cadd(lt, ls[c]), Ef * Ef);
            aa.lw[c][idx] = cadd(cscale(lt, Ef * dt / T(3)), cscale(ls[c], Ef * dt));
          }
          break;
        case ADJ3:   // lv += E ls ; lw = E dt lt/3 + dt/2 ls
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const C lt = aa.lt[c][idx];
            aa.lv[c][idx] = cadd(aa.lv[c][idx], cscale(ls[c], Ef));
            aa.lw[c][idx] = cadd(cscale(lt, Ef * dt / T(3)), cscale(ls[c], T(0.5) * dt));
          }
          break;
        case ADJ2:   // lv += E ls ; lw = E^2 dt lt/6 + E dt/2 ls
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const C lt = aa.lt[c][idx];
            aa.lv[c][idx] = cadd(aa.lv[c][idx], cscale(ls[c], Ef));
            aa.lw[c][idx] = cadd(cscale(lt, Ef * Ef * dt / T(6)), cscale(ls[c], T(0.5) * Ef * dt));
          }
          break;
        default:     // stage 1: lam = lv + ls
#pragma unroll
          for (int c = 0; c < 3; ++c) aa.lam[c][idx] = cadd(aa.lv[c][idx], ls[c]);
          break;
      }
    }
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
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long row = t / g.nxh;
    const int ix = (int)(t % g.nxh);
    const int iy = (int)(row % g.ny), iz = (int)(row / g.ny);
    const long long idx = row * g.nxp + ix;
    const double ky = wavenum(iy, g.ny), kz = wavenum(iz, g.nz);
    const double k2 = (double)ix * ix + ky * ky + kz * kz;
    if (ao.op == AO_INIT) {
      const bool cut = k2 >= ao.kcut2 && k2 > 0.0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const C l = cut ? czero<C>() : ao.in[c][idx];
        ao.out1[c][idx] = l;
        ao.out2[c][idx] = cscale(l, ao.dt / T(6));
      }
    } else {
      const int ll = (int)floor(sqrt(k2) + 0.5);
      const bool in = ll >= ao.kmin && ll <= ao.kmax;
      const T f = in ? (T)(2.0 * k2 * (ix == 0 ? 0.5 : 1.0)) : T(0);
#pragma unroll
      for (int c = 0; c < 3; ++c) ao.out1[c][idx] = cscale(ao.in[c][idx], f);
    }
  }
}

}  // namespace sc
