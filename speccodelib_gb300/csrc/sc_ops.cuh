// Elementwise spectral operators and FP64 reductions.
//
// These are the pieces of the reference's L3 layer that are not fused into
// the transform passes: the standalone operators behind the reference-
// signature entry points (projection.f90, symmetrize.f90, dealiasing.f90,
// force.f90), the seeded initial field's post-processing
// (initialize.f90:328-368) and the in-loop diagnostics
// (specdns-forced-omp-ft.f90:142-176).  All sums are accumulated in double.
#pragma once
#include "sc_passes.cuh"
#include "sc_rot.cuh"
#include "sc_ab2v.cuh"

namespace sc {

// ---------------------------------------------------------------------------
// reductions over spectral (or packed physical) fields
// ---------------------------------------------------------------------------
enum DiagQ { DQ_ENERGY = 0, DQ_K2Q = 1, DQ_MAXDIV = 2, DQ_NONFINITE = 3, DQ_MAXU2 = 4, DQ_N = 5 };

template <typename T> struct DiagArgs {
  const C2<T>* v[3];
  int physical;           // 0: spectral fields (energy etc.); 1: packed physical rows (max |u|^2)
  double kmax2;           // < 0: every mode; else only modes with k2 < kmax2 (forcing band)
  int rows_per_block;
  int nshell;             // 0: no spectrum; else nx/2 shells
  double* partial;        // [gridDim.x][DQ_N + nshell]
  double* out;            // [DQ_N + nshell]
  int nblocks;
  int shell_lo, shell_hi; // shell_hi > 0: only shells lo..hi (floor(|k| + 1/2))
};

template <typename T>
__global__ void __launch_bounds__(256) diag_partial_kernel(DiagArgs<T> da, Geom g) {
  using C = C2<T>;
  extern __shared__ double shells[];
  __shared__ double red[8 + 1];
  const int ns = da.nshell;
  for (int i = threadIdx.x; i < ns; i += blockDim.x) shells[i] = 0.0;
  __syncthreads();
  // per-point products in the field's precision, sums in double
  double e = 0.0, k2q = 0.0, nf = 0.0;
  T mdiv = T(0), mu2 = T(0);
  const long long rows = (long long)g.ny * g.nz;
  const long long r0 = (long long)blockIdx.x * da.rows_per_block;
  const long long r1 = r0 + da.rows_per_block < rows ? r0 + da.rows_per_block : rows;
  const int ncol = da.physical ? g.nx / 2 : g.nxh;
  const bool kmax_on = da.kmax2 >= 0.0;
  const int kmax_b = k2_lt(da.kmax2);
  for (Walk3 w(r0 * ncol + threadIdx.x, blockDim.x, r1 * ncol, ncol, g.ny); w.ok(); w.next()) {
    const int ix = w.ix;
    const long long idx = w.row() * g.nxp + ix;
    const C a = da.v[0][idx], b = da.v[1][idx], c = da.v[2][idx];
    if (da.physical) {
      const T ue = a.x * a.x + b.x * b.x + c.x * c.x;
      const T uo = a.y * a.y + b.y * b.y + c.y * c.y;
      mu2 = fmax(mu2, fmax(ue, uo));
      if (!isfinite(ue) || !isfinite(uo)) nf += 1.0;
      continue;
    }
    const int kyi = wavenum(w.iy, g.ny), kzi = wavenum(w.iz, g.nz);
    const int k2 = ix * ix + kyi * kyi + kzi * kzi;
    if (kmax_on && !(k2 < kmax_b)) continue;
    const int ll = (da.shell_hi > 0 || ns > 0) ? shell_index(k2) : 0;
    if (da.shell_hi > 0 && (ll < da.shell_lo || ll > da.shell_hi)) continue;
    T q = a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y + c.x * c.x + c.y * c.y;
    if (!isfinite(q)) nf += 1.0;
    if (ix == 0) q *= T(0.5);
    e += (double)q;
    k2q += (double)((T)k2 * q);
    const T kx = (T)ix, ky = (T)kyi, kz = (T)kzi;
    const T dr = kx * a.x + ky * b.x + kz * c.x, di = kx * a.y + ky * b.y + kz * c.y;
    mdiv = fmax(mdiv, sqrt(dr * dr + di * di));
    if (ns > 0 && ll >= 1 && ll <= ns) atomicAdd(&shells[ll - 1], (double)q);
  }
  double* out = da.partial + (long long)blockIdx.x * (DQ_N + ns);
  double s;
  s = block_sum<256>(e, red);
  if (threadIdx.x == 0) out[DQ_ENERGY] = s;
  s = block_sum<256>(k2q, red);
  if (threadIdx.x == 0) out[DQ_K2Q] = s;
  s = block_sum<256>(nf, red);
  if (threadIdx.x == 0) out[DQ_NONFINITE] = s;
  // maxima: reuse the sum tree with max
  double m1 = warp_max((double)mdiv), m2 = warp_max((double)mu2);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = m1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int i = 0; i < 8; ++i) m = fmax(m, red[i]);
    out[DQ_MAXDIV] = m;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { red[threadIdx.x >> 5] = m2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int i = 0; i < 8; ++i) m = fmax(m, red[i]);
    out[DQ_MAXU2] = m;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ns; i += blockDim.x) out[DQ_N + i] = shells[i];
}

// Column-wise reduction of the block partials in block order (deterministic).
static __global__ void diag_final_kernel(const double* partial, int nblocks, int ncols, double* out) {
  for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
    double s = 0.0;
    const bool isMax = (c == DQ_MAXDIV || c == DQ_MAXU2);
    for (int b = 0; b < nblocks; ++b) {
      const double x = partial[(long long)b * ncols + c];
      s = isMax ? fmax(s, x) : s + x;
    }
    out[c] = s;
  }
}

// ---------------------------------------------------------------------------
// elementwise spectral operators
// ---------------------------------------------------------------------------
enum SpecOp {
  OP_PROJECT = 0,       // projection.f90:16-30 on fields 0..2
  OP_ZERO_PLANES = 1,   // symmetrize.f90:43-49 on fields 0..n-1
  OP_KX0_COPY = 2,      // symmetrize.f90:52-62 (after OP_ZERO_PLANES)
  OP_MASK = 3,          // zero k2 >= kcut2 (dealiasing.f90:35, dns-deform.f90:233-237)
  OP_FORCE_ADD = 4,     // force.f90:24-29: f[0..2] += a * g[0..2] on k2 < fkmax2
  OP_INIT_SHAPE = 5,    // initialize.f90:328-332 projection with +tiny
  OP_INIT_AMP = 6,      // initialize.f90:349-360 amplitude (akp) or k^(-11/6) band
  OP_SCALE = 7,         // f *= scalar (scalar from device or host value)
  OP_AXPBY = 8,         // f[c] = alpha f[c] + beta g[c]
  OP_PMUL = 9,          // packed physical rows: f[c] = (f[c].x g0.x, f[c].y g0.y) (convecphi_dns.f90:23)
  OP_IDIV = 10,         // f[0] = a i (kx f0 + ky f1 + kz f2) (convecphi_dns.f90:25-45)
  OP_FORCE_BAND = 11,   // force_rot.f90:24-28: f[0..n-1] += a g[0..n-1] on b <= k2 < kcut2
  OP_DX = 12,           // f[0] = i kx f[0] (skewness.f90:17-21)
  OP_CURL = 13,         // f[0..2] = i k x f[0..2] (enstrophy.f90:16-18)
  OP_HERMITIANIZE = 14  // hermitianize.f90:10-22: the kx = 0 copy of OP_KX0_COPY, ky = -ny/2 row included
};

template <typename T> struct SpecOpArgs {
  int op;
  int nfields;
  C2<T>* f[6];
  const C2<T>* gsrc[3];
  double a, b;            // scalars
  const double* dscal;    // device scalar (OP_SCALE: multiply by sqrt(a / *dscal) if set)
  double kcut2;
  double akp, u0, kmin, kmax;
  int spectrum_kind;      // 0: akp shape, 1: k^(-11/6) band
};

template <typename T>
__global__ void __launch_bounds__(256) specop_kernel(SpecOpArgs<T> oa, Geom g) {
  using C = C2<T>;
  const long long rows = (long long)g.ny * g.nz;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long tstride = (long long)gridDim.x * blockDim.x;
  T sfac = T(1);
  if (oa.op == OP_SCALE) sfac = oa.dscal ? (T)sqrt(oa.a / *oa.dscal) : (T)oa.a;
  if (oa.op == OP_KX0_COPY || oa.op == OP_HERMITIANIZE) {
    // destinations (iz > nz/2, or the line iz = 0, iy > ny/2) never serve as sources
    const bool zero_nyq = oa.op == OP_KX0_COPY;   // after OP_ZERO_PLANES that row's sources are zero
    for (long long t = t0; t < rows; t += tstride) {
      const int iy = (int)(t % g.ny), iz = (int)(t / g.ny);
      if (!(iz > g.nz / 2 || (iz == 0 && iy > g.ny / 2))) continue;
      const int sy = (g.ny - iy) % g.ny, sz = (g.nz - iz) % g.nz;
      const long long d = ((long long)iz * g.ny + iy) * g.nxp, s = ((long long)sz * g.ny + sy) * g.nxp;
      for (int c = 0; c < oa.nfields; ++c)
        oa.f[c][d] = (zero_nyq && iy == g.ny / 2) ? czero<C>() : cconj(oa.f[c][s]);
    }
    return;
  }
  const int kc_b = k2_lt(oa.kcut2), b_b = k2_lt(oa.b);
  for (Walk3 w(t0, tstride, rows * g.nxh, g.nxh, g.ny); w.ok(); w.next()) {
    const int ix = w.ix, iy = w.iy, iz = w.iz;
    const long long idx = w.row() * g.nxp + ix;
    const int kyi = wavenum(iy, g.ny), kzi = wavenum(iz, g.nz);
    const int k2i = ix * ix + kyi * kyi + kzi * kzi;
    const T kx = (T)ix, ky = (T)kyi, kz = (T)kzi;
    switch (oa.op) {
      case OP_PROJECT:
      case OP_INIT_SHAPE: {
        C w0 = oa.f[0][idx], w1 = oa.f[1][idx], w2 = oa.f[2][idx];
        if (k2i > 0) {
          C tt = cadd(cadd(cscale(w0, kx), cscale(w1, ky)), cscale(w2, kz));
          tt = cscale(tt, T(1) / (T)k2i);
          w0 = csub(w0, cscale(tt, kx));
          w1 = csub(w1, cscale(tt, ky));
          w2 = csub(w2, cscale(tt, kz));
        }
        oa.f[0][idx] = w0; oa.f[1][idx] = w1; oa.f[2][idx] = w2;
        break;
      }
      case OP_ZERO_PLANES:
        if (iy == g.ny / 2 || iz == g.nz / 2 || ix == g.nxh - 1 || (ix == 0 && iy == 0 && iz == 0))
          for (int c = 0; c < oa.nfields; ++c) oa.f[c][idx] = czero<C>();
        break;
      case OP_MASK:
        if (k2i >= kc_b && k2i > 0)
          for (int c = 0; c < oa.nfields; ++c) oa.f[c][idx] = czero<C>();
        break;
      case OP_FORCE_ADD:
        // k2(1,1,1) = tiny < fkmax^2: the mean mode is in the band too
        if (k2i < kc_b) {
          const T a = (T)oa.a;
          for (int c = 0; c < 3; ++c) oa.f[c][idx] = cadd(oa.f[c][idx], cscale(oa.gsrc[c][idx], a));
        }
        break;
      case OP_INIT_AMP: {
        // k2 at the mean mode is tiny(1.0_sp) (wavenumber.f90:156)
        const double k2r = (k2i == 0) ? 1.1754943508222875e-38 : (double)k2i;
        double amp;
        if (oa.spectrum_kind == 0) {
          const double pi = 3.1415926536;
          amp = oa.u0 * sqrt(8.0 * sqrt(2.0 / pi) / (3.0 * pi * pow(oa.akp, 5.0))) * sqrt(k2r) *
                exp(-k2r / (oa.akp * oa.akp));
        } else {
          const double k = sqrt(k2r);
          amp = (k >= oa.kmin && k <= oa.kmax) ? pow(k, -11.0 / 6.0) : 0.0;
        }
        for (int c = 0; c < 3; ++c) oa.f[c][idx] = cscale(oa.f[c][idx], (T)amp);
        break;
      }
      case OP_SCALE:
        for (int c = 0; c < oa.nfields; ++c) oa.f[c][idx] = cscale(oa.f[c][idx], sfac);
        break;
      case OP_AXPBY:
        for (int c = 0; c < oa.nfields; ++c)
          oa.f[c][idx] = cadd(cscale(oa.f[c][idx], (T)oa.a), cscale(oa.gsrc[c][idx], (T)oa.b));
        break;
      case OP_PMUL: {
        const C gp = oa.gsrc[0][idx];
        for (int c = 0; c < oa.nfields; ++c) {
          const C fp = oa.f[c][idx];
          oa.f[c][idx] = mk<C>(fp.x * gp.x, fp.y * gp.y);
        }
        break;
      }
      case OP_IDIV: {
        const C d = cadd(cadd(cscale(oa.f[0][idx], kx), cscale(oa.f[1][idx], ky)), cscale(oa.f[2][idx], kz));
        oa.f[0][idx] = cmuli(cscale(d, (T)oa.a));
        break;
      }
      case OP_DX:
        oa.f[0][idx] = cmuli(cscale(oa.f[0][idx], kx));
        break;
      case OP_CURL: {
        const C u0 = oa.f[0][idx], u1 = oa.f[1][idx], u2 = oa.f[2][idx];
        oa.f[0][idx] = cmuli(csub(cscale(u2, ky), cscale(u1, kz)));
        oa.f[1][idx] = cmuli(csub(cscale(u0, kz), cscale(u2, kx)));
        oa.f[2][idx] = cmuli(csub(cscale(u1, kx), cscale(u0, ky)));
        break;
      }
      case OP_FORCE_BAND:
        if (k2i < kc_b && !(k2i < b_b)) {
          const T a = (T)oa.a;
          for (int c = 0; c < oa.nfields; ++c) oa.f[c][idx] = cadd(oa.f[c][idx], cscale(oa.gsrc[c][idx], a));
        }
        break;
      default:
        break;
    }
  }
}


// ---------------------------------------------------------------------------
// force_rot.f90's coefficient on the device: a = eps / (2 kinet + tiny), kinet
// the 1/2-weighted (kx = 0) energy of v on lo2 <= k2 < hi2 (force_rot.f90:
// 16-27).  One block walks the band's bounding box |k_i| <= floor(sqrt(hi2))
// in a fixed order and sums in FP64, so the result is deterministic and no
// host synchronisation is needed (the rotating pass reads *out in its
// z-forward epilogue).
// ---------------------------------------------------------------------------
template <typename T> struct BandArgs {
  const C2<T>* v[3];
  double lo2, hi2, eps, tiny;
  double* out;
};

template <typename T>
__global__ void __launch_bounds__(256) band_coef_kernel(BandArgs<T> ba, Geom g) {
  __shared__ double red[256 / 32 + 1];
  const int lo_b = k2_lt(ba.lo2), hi_b = k2_lt(ba.hi2);
  int kb = 0;
  while ((kb + 1) * (kb + 1) < hi_b) ++kb;   // largest |k_i| with k_i^2 < hi2
  const int nkx = min(kb, g.nxh - 1) + 1;
  const int ky0 = max(-kb, -g.ny / 2), ky1 = min(kb, g.ny / 2 - 1);
  const int kz0 = max(-kb, -g.nz / 2), kz1 = min(kb, g.nz / 2 - 1);
  const int nky = ky1 - ky0 + 1, nkz = kz1 - kz0 + 1;
  const long long total = (long long)nkx * nky * nkz;
  double q = 0.0;
  for (long long t = threadIdx.x; t < total; t += blockDim.x) {
    const int ix = (int)(t % nkx);
    const int ky = ky0 + (int)((t / nkx) % nky);
    const int kz = kz0 + (int)(t / ((long long)nkx * nky));
    const int k2 = ix * ix + ky * ky + kz * kz;
    if (k2 < lo_b || k2 >= hi_b) continue;
    const int iy = ky < 0 ? ky + g.ny : ky, iz = kz < 0 ? kz + g.nz : kz;
    const long long idx = ((long long)iz * g.ny + iy) * g.nxp + ix;
    double e = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const C2<T> a = ba.v[c][idx];
      e += (double)a.x * a.x + (double)a.y * a.y;
    }
    q += ix == 0 ? 0.5 * e : e;
  }
  const double kinet = block_sum<256>(q, red);
  if (threadIdx.x == 0) *ba.out = ba.eps / (2.0 * kinet + ba.tiny);
}

// ---------------------------------------------------------------------------
// helical-wave AB2 update of the rotating solver (rot_point, sc_rot.cuh)
// ---------------------------------------------------------------------------
template <typename T> struct RotArgs {
  int pass;              // 0: Euler half step, 1: midpoint restart, >= 2: AB2
  C2<T>* v[3];           // velocity: read at pass 0, rewritten every pass
  const C2<T>* w[3];     // right-hand side of this pass
  C2<T>* o[3];           // previous right-hand side (written at pass 0 and >= 2)
  C2<T>* a[2];           // helical amplitudes a+, a-
  double nu, dt, om;     // viscosity, time step, rotation rate
  double kcut2;          // v = 0 where k2 >= kcut2 (when mask_v)
  int mask_v;            // truncate the rebuilt velocity
  // passive scalar (when phi is set): phi, its right-hand side, the previous
  // right-hand side (written at pass 0 and >= 2), the initial phi (written at
  // pass 0, read at pass 1); Prandtl number pr
  C2<T>* phi;
  const C2<T>* wphi;
  C2<T>* ophi;
  C2<T>* phi0;
  double pr;
};

template <typename T>
__global__ void __launch_bounds__(256) rot_update_kernel(RotArgs<T> ra, Geom g) {
  using C = C2<T>;
  const long long rows = (long long)g.ny * g.nz;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long tstride = (long long)gridDim.x * blockDim.x;
  const int kc_b = k2_lt(ra.kcut2);
  const T nu = (T)ra.nu, dt = (T)ra.dt, om = (T)ra.om;
  const int pass = ra.pass;
  for (Walk3 it(t0, tstride, rows * g.nxh, g.nxh, g.ny); it.ok(); it.next()) {
    const long long idx = it.row() * g.nxp + it.ix;
    const int ky = wavenum(it.iy, g.ny), kz = wavenum(it.iz, g.nz);
    const int k2 = it.ix * it.ix + ky * ky + kz * kz;
    Cx<T> v[3], w[3], o[3], ap = cx(T(0), T(0)), am = cx(T(0), T(0));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const C wc = ra.w[c][idx];
      w[c] = cx(wc.x, wc.y);
      v[c] = o[c] = cx(T(0), T(0));
      if (pass == 0) {
        const C vc = ra.v[c][idx];
        v[c] = cx(vc.x, vc.y);
      }
      if (pass >= 2) {
        const C oc = ra.o[c][idx];
        o[c] = cx(oc.x, oc.y);
      }
    }
    if (pass > 0) {
      const C a0 = ra.a[0][idx], a1 = ra.a[1][idx];
      ap = cx(a0.x, a0.y);
      am = cx(a1.x, a1.y);
    }
    rot_point<T>(pass, it.ix, ky, kz, ra.mask_v && k2 >= kc_b, nu, dt, om, v, w, o, ap, am);
    if (ra.phi) {
      const C p = ra.phi[idx], wp = ra.wphi[idx];
      Cx<T> ph = cx(p.x, p.y), op = cx(T(0), T(0)), p0 = cx(T(0), T(0));
      if (pass >= 2) {
        const C q = ra.ophi[idx];
        op = cx(q.x, q.y);
      }
      if (pass == 1) {
        const C q = ra.phi0[idx];
        p0 = cx(q.x, q.y);
      }
      rot_scalar_point<T>(pass, k2, nu, dt, (T)ra.pr, ph, cx(wp.x, wp.y), op, p0);
      ra.phi[idx] = mk<C>(ph.re, ph.im);
      if (pass != 1) ra.ophi[idx] = mk<C>(op.re, op.im);
      if (pass == 0) ra.phi0[idx] = mk<C>(p0.re, p0.im);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      ra.v[c][idx] = mk<C>(v[c].re, v[c].im);
      if (pass != 1) ra.o[c][idx] = mk<C>(o[c].re, o[c].im);
    }
    ra.a[0][idx] = mk<C>(ap.re, ap.im);
    ra.a[1][idx] = mk<C>(am.re, am.im);
  }
}

// ---------------------------------------------------------------------------
// variable-step IF-AB2 update (ab2v_point, sc_ab2v.cuh)
// ---------------------------------------------------------------------------
template <typename T> struct Ab2vArgs {
  int pass;              // 0: Euler step, 1: restart from v0, >= 2: AB2
  C2<T>* v[3];           // velocity, rewritten every pass
  const C2<T>* w[3];     // right-hand side of this pass
  C2<T>* o[3];           // previous right-hand side (written at pass 0 and >= 2)
  C2<T>* v0[3];          // initial field (written at pass 0, read at pass 1)
  double nu, dt, dto;    // viscosity, this step, the previous step
  double s, ek, dl;      // the pass's weights
  double kcut2;          // v = 0 where k2 >= kcut2 and at the mean mode (when mask_v)
  int mask_v;
  // passive scalar (when phi is set): phi, its right-hand side, its history,
  // the initial phi; Prandtl number; hist_rhs: history at pass 0 is wphi
  C2<T>* phi;
  const C2<T>* wphi;
  C2<T>* ophi;
  C2<T>* phi0;
  double pr;
  int hist_rhs;
};

template <typename T>
__global__ void __launch_bounds__(256) ab2v_update_kernel(Ab2vArgs<T> aa, Geom g) {
  using C = C2<T>;
  const long long rows = (long long)g.ny * g.nz;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long tstride = (long long)gridDim.x * blockDim.x;
  const int kc_b = k2_lt(aa.kcut2);
  const T nu = (T)aa.nu, dt = (T)aa.dt, dto = (T)aa.dto, s = (T)aa.s, ek = (T)aa.ek, dl = (T)aa.dl;
  const int pass = aa.pass;
  for (Walk3 it(t0, tstride, rows * g.nxh, g.nxh, g.ny); it.ok(); it.next()) {
    const long long idx = it.row() * g.nxp + it.ix;
    const int ky = wavenum(it.iy, g.ny), kz = wavenum(it.iz, g.nz);
    const int k2 = it.ix * it.ix + ky * ky + kz * kz;
    Cx<T> v[3], w[3], o[3], v0[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const C vc = aa.v[c][idx], wc = aa.w[c][idx];
      v[c] = cx(vc.x, vc.y);
      w[c] = cx(wc.x, wc.y);
      o[c] = v0[c] = cx(T(0), T(0));
      if (pass >= 2) {
        const C oc = aa.o[c][idx];
        o[c] = cx(oc.x, oc.y);
      }
      if (pass == 1) {
        const C zc = aa.v0[c][idx];
        v0[c] = cx(zc.x, zc.y);
      }
    }
    ab2v_point<T>(pass, k2, aa.mask_v && (k2 >= kc_b || k2 == 0), nu, dt, dto, s, ek, dl, v, w, o, v0);
    if (aa.phi) {
      const C p = aa.phi[idx], wp = aa.wphi[idx];
      Cx<T> ph = cx(p.x, p.y), op = cx(T(0), T(0)), p0 = cx(T(0), T(0));
      if (pass >= 2) {
        const C q = aa.ophi[idx];
        op = cx(q.x, q.y);
      }
      if (pass == 1) {
        const C q = aa.phi0[idx];
        p0 = cx(q.x, q.y);
      }
      ab2v_scalar_point<T>(pass, k2, aa.hist_rhs != 0, nu, dt, dto, (T)aa.pr, s, ek, dl, ph, cx(wp.x, wp.y), op, p0);
      aa.phi[idx] = mk<C>(ph.re, ph.im);
      if (pass != 1) aa.ophi[idx] = mk<C>(op.re, op.im);
      if (pass == 0) aa.phi0[idx] = mk<C>(p0.re, p0.im);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      aa.v[c][idx] = mk<C>(v[c].re, v[c].im);
      if (pass != 1) aa.o[c][idx] = mk<C>(o[c].re, o[c].im);
      if (pass == 0) aa.v0[c][idx] = mk<C>(v0[c].re, v0[c].im);
    }
  }
}

// ---------------------------------------------------------------------------
// post-processing on physical fields held as packed rows (x = 2m in .x,
// x = 2m+1 in .y, m < nx/2)
// ---------------------------------------------------------------------------
// Sums of d^2 and d^3 over the real points, FP64, block partials
// partial[b*2 + {0, 1}] (skewness.f90:22-45).
template <typename T>
__global__ void __launch_bounds__(256) moments_kernel(const C2<T>* d, Geom g, int rows_per_block, double* partial) {
  __shared__ double red[256 / 32 + 1];
  const long long rows = (long long)g.ny * g.nz;
  const long long r0 = (long long)blockIdx.x * rows_per_block;
  const long long r1 = r0 + rows_per_block < rows ? r0 + rows_per_block : rows;
  const int m = g.nx / 2;
  double s2 = 0.0, s3 = 0.0;
  for (long long row = r0; row < r1; ++row)
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      const C2<T> v = d[row * g.nxp + i];
      const double a = v.x, b = v.y;
      s2 += a * a + b * b;
      s3 += a * a * a + b * b * b;
    }
  s2 = block_sum<256>(s2, red);
  s3 = block_sum<256>(s3, red);
  if (threadIdx.x == 0) {
    partial[2 * (long long)blockIdx.x] = s2;
    partial[2 * (long long)blockIdx.x + 1] = s3;
  }
}

// Block partials summed in block order (deterministic): out[0..1].
static __global__ void moments_final_kernel(const double* partial, int nblocks, double* out) {
  if (threadIdx.x < 2) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += partial[2 * (long long)b + threadIdx.x];
    out[threadIdx.x] = s;
  }
}

// Enstrophy density 1/2 |w|^2 of three physical vorticity fields into a real
// (nz, ny, nx) array, FP64 (enstrophy.f90:24-34).
template <typename T>
__global__ void __launch_bounds__(256) enstrophy_kernel(const C2<T>* w0, const C2<T>* w1, const C2<T>* w2, Geom g,
                                                        double* out) {
  const int m = g.nx / 2;
  const long long total = (long long)g.ny * g.nz * m;
  for (Walk3 w(blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x, total, m, g.ny);
       w.ok(); w.next()) {
    const long long row = w.row();
    const int i = w.ix;
    const long long idx = row * g.nxp + i;
    const C2<T> a = w0[idx], b = w1[idx], c = w2[idx];
    out[row * g.nx + 2 * i] = 0.5 * ((double)a.x * a.x + (double)b.x * b.x + (double)c.x * c.x);
    out[row * g.nx + 2 * i + 1] = 0.5 * ((double)a.y * a.y + (double)b.y * b.y + (double)c.y * c.y);
  }
}

// ---------------------------------------------------------------------------
// strain rate in spectral space: S_ij = i (k_i v_j + k_j v_i)/2, order
// 11 12 13 22 23 33 (smag.f90:21-32)
// ---------------------------------------------------------------------------
template <typename T> struct StrainArgs {
  const C2<T>* v[3];
  C2<T>* s[6];
};

template <typename T>
__global__ void __launch_bounds__(256) strain_kernel(StrainArgs<T> sa, Geom g) {
  using C = C2<T>;
  const long long total = (long long)g.ny * g.nz * g.nxh;
  const T half = T(0.5);
  for (Walk3 w(blockIdx.x * (long long)blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x, total, g.nxh,
               g.ny);
       w.ok(); w.next()) {
    const int ix = w.ix;
    const long long idx = w.row() * g.nxp + ix;
    const T kx = (T)ix, ky = (T)wavenum(w.iy, g.ny), kz = (T)wavenum(w.iz, g.nz);
    const C v0 = sa.v[0][idx], v1 = sa.v[1][idx], v2 = sa.v[2][idx];
    sa.s[0][idx] = cmuli(cscale(v0, kx));
    sa.s[1][idx] = cmuli(cscale(cadd(cscale(v1, kx), cscale(v0, ky)), half));
    sa.s[2][idx] = cmuli(cscale(cadd(cscale(v2, kx), cscale(v0, kz)), half));
    sa.s[3][idx] = cmuli(cscale(v1, ky));
    sa.s[4][idx] = cmuli(cscale(cadd(cscale(v2, ky), cscale(v1, kz)), half));
    sa.s[5][idx] = cmuli(cscale(v2, kz));
  }
}

// ---------------------------------------------------------------------------
// physical-space pointwise kernels on packed rows (x = 2m: .x, x = 2m+1: .y)
// ---------------------------------------------------------------------------
enum PhysOp {
  PH_TAU = 0,    // f[0..5] (S_ij) <- coef |S| S_ij, coef = -2 c1 delta^2 scale (smag.f90:41-64)
  PH_DYN1 = 1,   // dynamic procedure, first products (dynsmag.f90:43-48, 103-115, 133-145)
  PH_DYN2 = 2    // L_ij, M_ij and the box sums LM, MM (dynsmag.f90:71-76, 163-184)
};

template <typename T> struct PhysArgs {
  int op;
  C2<T>* f[24];
  const double* c1;      // device scalar (c1 or cs2)
  double delta2, delta_test2;
  T scale;               // 1/(nx ny nz)
  double* partial;       // PH_DYN2: [nblocks][2] (LM, MM)
  int rows_per_block;
};

template <typename R>
__device__ __forceinline__ R smag_abs(R s11, R s12, R s13, R s22, R s23, R s33) {
  return sqrt(R(2) * (s11 * s11 + s22 * s22 + s33 * s33 + R(2) * (s12 * s12 + s13 * s13 + s23 * s23)));
}

template <typename T>
__global__ void __launch_bounds__(256) phys_kernel(PhysArgs<T> pa, Geom g) {
  using C = C2<T>;
  __shared__ double red[9];
  const long long rows = (long long)g.ny * g.nz;
  const int ncol = g.nx / 2;
  const long long r0 = (long long)blockIdx.x * pa.rows_per_block;
  const long long r1 = r0 + pa.rows_per_block < rows ? r0 + pa.rows_per_block : rows;
  double lm = 0.0, mm = 0.0;
  T coef = T(0);
  if (pa.op == PH_TAU) coef = (T)(-2.0 * (*pa.c1) * pa.delta2) * pa.scale;
  for (Walk3 w(r0 * ncol + threadIdx.x, blockDim.x, r1 * ncol, ncol, g.ny); w.ok(); w.next()) {
    const long long idx = w.row() * g.nxp + w.ix;
    if (pa.op == PH_TAU) {
      C s[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) s[q] = pa.f[q][idx];
      const T ar = smag_abs(s[0].x, s[1].x, s[2].x, s[3].x, s[4].x, s[5].x);
      const T ai = smag_abs(s[0].y, s[1].y, s[2].y, s[3].y, s[4].y, s[5].y);
#pragma unroll
      for (int q = 0; q < 6; ++q) pa.f[q][idx] = mk<C>(ar * s[q].x * coef, ai * s[q].y * coef);
    } else if (pa.op == PH_DYN1) {
      // slots: u 0-2, gu 3-5, S 6-11, gS 12-17, D 18-23
      C u[3], gu[3], s[6], gs[6];
#pragma unroll
      for (int q = 0; q < 3; ++q) { u[q] = pa.f[q][idx]; gu[q] = pa.f[3 + q][idx]; }
#pragma unroll
      for (int q = 0; q < 6; ++q) { s[q] = pa.f[6 + q][idx]; gs[q] = pa.f[12 + q][idx]; }
      const int ii[6] = {0, 0, 0, 1, 1, 2}, jj[6] = {0, 1, 2, 1, 2, 2};
      const T sc = pa.scale;
      const T ar = smag_abs(s[0].x, s[1].x, s[2].x, s[3].x, s[4].x, s[5].x);
      const T ai = smag_abs(s[0].y, s[1].y, s[2].y, s[3].y, s[4].y, s[5].y);
      const T gr = smag_abs(gs[0].x, gs[1].x, gs[2].x, gs[3].x, gs[4].x, gs[5].x);
      const T gi = smag_abs(gs[0].y, gs[1].y, gs[2].y, gs[3].y, gs[4].y, gs[5].y);
      const T c2 = (T)(2.0 * pa.delta2), ct2 = (T)(-2.0 * pa.delta_test2);
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const C a = u[ii[q]], b = u[jj[q]];
        pa.f[18 + q][idx] = mk<C>(a.x * b.x * sc, a.y * b.y * sc);           // u_i u_j / N^3
        const C ga = gu[ii[q]], gb = gu[jj[q]];
        pa.f[q][idx] = mk<C>(ga.x * gb.x, ga.y * gb.y);                       // (g u_i)(g u_j)
        pa.f[6 + q][idx] = mk<C>(c2 * (ar * s[q].x) * sc, c2 * (ai * s[q].y) * sc);   // 2 D^2 |S| S / N^3
        pa.f[12 + q][idx] = mk<C>(ct2 * (gr * gs[q].x), ct2 * (gi * gs[q].y));        // -2 Dt^2 |gS| gS
      }
    } else {
      // slots: G 0-5, filt(s) 6-11, T 12-17, filt(D) 18-23
      const T wq[6] = {T(1), T(2), T(2), T(1), T(2), T(1)};
#pragma unroll
      for (int q = 0; q < 6; ++q) {
        const C G = pa.f[q][idx], fs = pa.f[6 + q][idx], Tq = pa.f[12 + q][idx], fD = pa.f[18 + q][idx];
        // products in the field's precision, sums in double
        const T Lr = fD.x - G.x, Li = fD.y - G.y;
        const T Mr = fs.x + Tq.x, Mi = fs.y + Tq.y;
        lm += (double)(wq[q] * (Lr * Mr + Li * Mi));
        mm += (double)(wq[q] * (Mr * Mr + Mi * Mi));
      }
    }
  }
  if (pa.op == PH_DYN2) {
    double s1 = block_sum<256>(lm, red);
    if (threadIdx.x == 0) pa.partial[2 * blockIdx.x] = s1;
    double s2 = block_sum<256>(mm, red);
    if (threadIdx.x == 0) pa.partial[2 * blockIdx.x + 1] = s2;
  }
}

// cs2 = LM/MM from the block partials in block order (dynsmag.f90:186).
static __global__ void dyn_final_kernel(const double* partial, int nblocks, double* c1, double* lm_mm) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double lm = 0.0, mm = 0.0;
  for (int b = 0; b < nblocks; ++b) { lm += partial[2 * b]; mm += partial[2 * b + 1]; }
  lm_mm[0] = lm;
  lm_mm[1] = mm;
  *c1 = lm / mm;
}

}  // namespace sc
