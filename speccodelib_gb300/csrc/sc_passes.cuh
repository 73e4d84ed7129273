// Pass kernels of the spectral Navier-Stokes right-hand side.
//
// One right-hand-side evaluation (the reference's ratesdudt,
// dns-deform.f90:259-288, around convec_dns.f90:1-55) is five passes over HBM:
//
//   zinv  (z-axis c2c, inverse)  reads the stage input v^ (3 fields), builds
//          v^ and w^ = i k x v^ (and S_ij for LES) on the fly, transforms along
//          kz, writes 6 (12) fields; also sums the forcing band energy K_f.
//   ypass (y-axis c2c)           in place on 6 (12) fields.
//   xpass (x-axis c2r, product, r2c)
//          per grid row: half-complex -> packed reals, u x w * 1/N^3 (and
//          tau_ij = -2 c1 D^2 |S| S_ij / N^3), packed reals -> half-complex.
//   ypass (y-axis c2c, forward)  in place on 3 (9) fields.
//   zfwd  (z-axis c2c, forward) + the whole spectral update: SGS divergence,
//          forcing, symmetrize, projection, 2/3 mask and the RK stage, then
//   fixup (kx = 0 plane) finishes the Hermitian copy of symmetrize.f90:52-62.
#pragma once
#include "sc_fft.cuh"
#include "sc_ab2v.cuh"

namespace sc {

template <typename T> struct Tile;
template <> struct Tile<float> { static constexpr int P = 16; };   // 128 B rows
template <> struct Tile<double> { static constexpr int P = 8; };   // 128 B rows

// Strided-axis tile: P pencils (consecutive kx) x N points, one radix-8 job
// per thread, 2 blocks per SM.  Long pencils use 8-wide tiles (64 B row
// segments, two full DRAM sectors) so a thread holds one job.
template <typename T, int LOGN> struct PencilCfg {
  static constexpr int N = 1 << LOGN;
  static constexpr int P = (sizeof(T) == 4 && LOGN < 9) ? 16 : 8;
  static constexpr int NT_RAW = P * N / 8;
  static constexpr int NT = NT_RAW > 512 ? 512 : (NT_RAW < 32 ? 32 : NT_RAW);
  static constexpr int MINB = NT >= 512 ? 2 : 4;
  static constexpr int MINB_FUSED = NT >= 512 ? 1 : 2;   // zinv/zfwd hold 3 fields
  using Engine = FFTEngine<T, LOGN, P, P, NT, true>;
  static constexpr size_t SMEM = sizeof(C2<T>) * Engine::SMEM_ELEMS;
};

// ---------------------------------------------------------------------------
// deterministic block reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// Sum over the block in a fixed order; result valid in thread 0.
template <int NT> __device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < (NT + 31) / 32; ++i) s += red[i];
  }
  return s;
}

// ---------------------------------------------------------------------------
// generic strided-axis pass (y or z), in place, nfields fields
// mode 0: plain; mode 1: z-pass with sharp filter k2 <= kmax2 and a scale
// applied to the input (test filter of dynsmag.f90:57-62)
// ---------------------------------------------------------------------------
template <typename T> struct PlainArgs {
  int nfields;
  long long axis_stride;   // elements between points of a pencil
  long long outer_stride;  // elements between blockIdx.y slabs
  int filter;              // 1: multiply input by scale*[k2 <= kmax2] (z-pass)
  double kmax2;
  T scale;
};

template <typename T, int LOGN, bool INV>
__global__ void __launch_bounds__(PencilCfg<T, LOGN>::NT, PencilCfg<T, LOGN>::MINB)
pencil_plain_kernel(FieldList<T> fl, PlainArgs<T> pa, Geom g, const C2<T>* __restrict__ tw) {
  using Cfg = PencilCfg<T, LOGN>;
  using E = typename Cfg::Engine;
  using C = C2<T>;
  constexpr int P = Cfg::P;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const int kx0 = blockIdx.x * P;
  const int nvalid = min(P, g.nxh - kx0);
  const long long base = (long long)blockIdx.y * pa.outer_stride + kx0;
  const int kyv = wavenum(blockIdx.y, g.ny);
  const int kmax_b = k2_le(pa.kmax2);
  for (int f = 0; f < pa.nfields; ++f) {
    C* __restrict__ fp = fl.f[f] + base;
    C in[E::J1][E::R1], out[E::JL][E::RL];
#pragma unroll
    for (int a = 0; a < E::J1; ++a)
#pragma unroll
      for (int r = 0; r < E::R1; ++r) {
        int p, n;
        bool ok = E::in_pos(a, r, p, n) && p < nvalid;
        C x = ok ? fp[n * pa.axis_stride + p] : czero<C>();
        if (pa.filter) {
          const int kx = kx0 + p, kz = wavenum(n, g.nz);
          x = (kx * kx + kyv * kyv + kz * kz < kmax_b) ? cscale(x, pa.scale) : czero<C>();
        }
        in[a][r] = x;
      }
    E::template run<INV>(in, out, sm, tw);
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        if (E::out_pos(a, r, p, n) && p < nvalid) fp[n * pa.axis_stride + p] = out[a][r];
      }
  }
}

// ---------------------------------------------------------------------------
// zinv: z-axis inverse pass generating the physical-space operands from v^
// ---------------------------------------------------------------------------
enum ZvMode { ZV_DNS = 0, ZV_SMAG = 1, ZV_DYN = 2, ZV_ADJ = 3 };
template <int MODE> struct ZvOut;
template <> struct ZvOut<ZV_DNS> { static constexpr int n = 6; };
template <> struct ZvOut<ZV_SMAG> { static constexpr int n = 12; };
template <> struct ZvOut<ZV_DYN> { static constexpr int n = 18; };
template <> struct ZvOut<ZV_ADJ> { static constexpr int n = 6; };   // + 3 adjoint outputs

struct ForceSum {
  int enabled;
  double fkmax2;
  double* partial;   // [tile * ny + iy]
};

template <typename T> struct ZvArgs {
  const C2<T>* v[3];
  ForceSum fs;
  double ktest2;     // ZV_DYN: test filter k2 <= ktest2
  // ZV_ADJ: adjoint of the right-hand side at stage input v, for the RHS
  // adjoint lam (kx = 0 copies already transposed): outputs 6..8 are
  // phi^ = D (zero P lam) / (2 N^3), D = 2 on the kx = 0 and kx = nx/2 planes.
  const C2<T>* lam[3];
  double* cpartial;  // forcing adjoint: sum over the band of Re(conj(mu) v)
  int mask_rhs;
  double kcut2;
  double inv_n3;
  int tiles_x;       // > 0: only the first tiles_x kx tiles (grid.x)
  int ustore;        // TMA z-inverse: u stored from its tiles by bulk tensor stores
};

// zero (symmetrize's planes and mean), optional RHS mask, then projection:
// mu = zero P lam at wavenumber (ix, ky, kz); kcut_b = k2_lt(kcut2).
template <typename C, typename R>
__device__ __forceinline__ void adj_mu(C* m, int ix, int iy, int iz, const Geom& g, int mask_rhs,
                                       int kcut_b) {
  const int kyi = wavenum(iy, g.ny), kzi = wavenum(iz, g.nz);
  const int k2i = ix * ix + kyi * kyi + kzi * kzi;
  const R kx = (R)ix, ky = (R)kyi, kz = (R)kzi;
  const R k2 = (R)k2i;
  const bool zero = iy == g.ny / 2 || iz == g.nz / 2 || ix == g.nxh - 1 || (ix == 0 && iy == 0 && iz == 0) ||
                    (mask_rhs && k2i >= kcut_b);
  if (zero) {
    m[0] = m[1] = m[2] = czero<C>();
    return;
  }
  if (k2 > R(0)) {
    C t = cadd(cadd(cscale(m[0], kx), cscale(m[1], ky)), cscale(m[2], kz));
    t = cscale(t, R(1) / k2);
    m[0] = csub(m[0], cscale(t, kx));
    m[1] = csub(m[1], cscale(t, ky));
    m[2] = csub(m[2], cscale(t, kz));
  }
}

// Output field `f` of the generator at wavenumber (kx, ky, kz).
//   ZV_DNS : v (3), w = i k x v (3)                      dns-deform.f90:265-273
//   ZV_SMAG: + S_ij, order 11 12 13 22 23 33             smag.f90:21-32
//   ZV_DYN : u (3), g u (3), S_ij (6), g S_ij (6)        dynsmag.f90:29-34,80-93
template <int MODE, typename C, typename R>
__device__ __forceinline__ C zv_gen(int f, C v0, C v1, C v2, R kx, R ky, R kz, bool gin) {
  const R half = R(0.5);
  const C v[3] = {v0, v1, v2};
  int q = f;
  if (MODE == ZV_DYN) {
    // fields: u (0-2), g u (3-5), S (6-11), g S (12-17)
    const bool filt = (f >= 3 && f < 6) || f >= 12;
    if (filt && !gin) return czero<C>();
    if (f < 6) {
      const int c = f % 3;
      return c == 0 ? v[0] : (c == 1 ? v[1] : v[2]);
    }
    q = 6 + (f - 6) % 6;
  }
  switch (q) {
    case 0: return v[0];
    case 1: return v[1];
    case 2: return v[2];
    case 3: return cmuli(csub(cscale(v[2], ky), cscale(v[1], kz)));
    case 4: return cmuli(csub(cscale(v[0], kz), cscale(v[2], kx)));
    case 5: return cmuli(csub(cscale(v[1], kx), cscale(v[0], ky)));
    case 6: return cmuli(cscale(v[0], kx));
    case 7: return cmuli(cscale(cadd(cscale(v[1], kx), cscale(v[0], ky)), half));
    case 8: return cmuli(cscale(cadd(cscale(v[2], kx), cscale(v[0], kz)), half));
    case 9: return cmuli(cscale(v[1], ky));
    case 10: return cmuli(cscale(cadd(cscale(v[2], ky), cscale(v[1], kz)), half));
    default: return cmuli(cscale(v[2], kz));
  }
}

template <typename T, int LOGN, int MODE>
__global__ void __launch_bounds__(PencilCfg<T, LOGN>::NT, PencilCfg<T, LOGN>::MINB_FUSED)
zinv_vel_kernel(ZvArgs<T> za, FieldList<T> out, Geom g, const C2<T>* __restrict__ tw) {
  using Cfg = PencilCfg<T, LOGN>;
  using E = typename Cfg::Engine;
  using C = C2<T>;
  constexpr int P = Cfg::P;
  constexpr int NT = Cfg::NT;
  constexpr int NOUT = ZvOut<MODE>::n;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  __shared__ double red[NT / 32 + 1];
  const int kx0 = blockIdx.x * P;
  const int iy = blockIdx.y;
  const int nvalid = min(P, g.nxh - kx0);
  const long long zstride = (long long)g.ny * g.nxp;
  const long long base = (long long)iy * g.nxp + kx0;
  const T ky = (T)wavenum(iy, g.ny);
  const int kyi = wavenum(iy, g.ny);
  const int fk_b = k2_lt(za.fs.fkmax2), kt_b = k2_le(za.ktest2), kc_b = k2_lt(za.kcut2);

  C vr[E::J1][E::R1][3];
  double q = 0.0;
  const bool fsum = za.fs.enabled && ((double)kx0 * kx0 + (double)ky * ky < za.fs.fkmax2);
#pragma unroll
  for (int a = 0; a < E::J1; ++a)
#pragma unroll
    for (int r = 0; r < E::R1; ++r) {
      int p, n;
      bool ok = E::in_pos(a, r, p, n) && p < nvalid;
#pragma unroll
      for (int c = 0; c < 3; ++c) vr[a][r][c] = ok ? za.v[c][base + n * zstride + p] : czero<C>();
      if (fsum && ok) {
        const int kx = kx0 + p, kz = wavenum(n, g.nz);
        if (kx * kx + kyi * kyi + kz * kz < fk_b) {
          double e = 0.0;
#pragma unroll
          for (int c = 0; c < 3; ++c)
            e += (double)vr[a][r][c].x * vr[a][r][c].x + (double)vr[a][r][c].y * vr[a][r][c].y;
          q += (kx0 + p == 0) ? 0.5 * e : e;
        }
      }
    }
  if (fsum) {
    double s = block_sum<NT>(q, red);
    if (threadIdx.x == 0) za.fs.partial[(long long)blockIdx.x * g.ny + iy] = s;
  }
  for (int f = 0; f < NOUT; ++f) {
    C in[E::J1][E::R1], o[E::JL][E::RL];
#pragma unroll
    for (int a = 0; a < E::J1; ++a)
#pragma unroll
      for (int r = 0; r < E::R1; ++r) {
        int p, n;
        E::in_pos(a, r, p, n);
        const int kzi = wavenum(n, g.nz);
        const T kx = (T)(kx0 + p), kz = (T)kzi;
        bool gin = true;
        if (MODE == ZV_DYN) gin = (kx0 + p) * (kx0 + p) + kyi * kyi + kzi * kzi < kt_b;
        in[a][r] = zv_gen<MODE == ZV_ADJ ? ZV_DNS : MODE>(f, vr[a][r][0], vr[a][r][1], vr[a][r][2], kx, ky, kz, gin);
      }
    E::template run<true>(in, o, sm, tw);
    C* __restrict__ fp = out.f[f] + base;
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        if (E::out_pos(a, r, p, n) && p < nvalid) fp[n * zstride + p] = o[a][r];
      }
  }
  if constexpr (MODE == ZV_ADJ) {
    // mu = zero P lam; the band sum c = sum Re(conj(mu) v) for the forcing
    // adjoint; outputs phi^ = D mu / (2 N^3)
    double q = 0.0;
#pragma unroll
    for (int a = 0; a < E::J1; ++a)
#pragma unroll
      for (int r = 0; r < E::R1; ++r) {
        int p, n;
        bool ok = E::in_pos(a, r, p, n) && p < nvalid;
        C m[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) m[c] = ok ? za.lam[c][base + n * zstride + p] : czero<C>();
        if (ok) adj_mu<C, T>(m, kx0 + p, iy, n, g, za.mask_rhs, kc_b);
        if (fsum && ok) {
          const int kx = kx0 + p, kz = wavenum(n, g.nz);
          if (kx * kx + kyi * kyi + kz * kz < fk_b)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const C sv = za.v[c][base + n * zstride + p];
              q += (double)m[c].x * sv.x + (double)m[c].y * sv.y;
            }
        }
        const int ix = kx0 + p;
        const T d = (T)((ix == 0 || ix == g.nxh - 1) ? za.inv_n3 : 0.5 * za.inv_n3);
#pragma unroll
        for (int c = 0; c < 3; ++c) vr[a][r][c] = cscale(m[c], d);
      }
    if (fsum) {
      double s2 = block_sum<NT>(q, red);
      if (threadIdx.x == 0) za.cpartial[(long long)blockIdx.x * g.ny + iy] = s2;
    }
    for (int c = 0; c < 3; ++c) {
      C in[E::J1][E::R1], o[E::JL][E::RL];
#pragma unroll
      for (int a = 0; a < E::J1; ++a)
#pragma unroll
        for (int r = 0; r < E::R1; ++r) in[a][r] = c == 0 ? vr[a][r][0] : (c == 1 ? vr[a][r][1] : vr[a][r][2]);
      E::template run<true>(in, o, sm, tw);
      C* __restrict__ fp = out.f[6 + c] + base;
#pragma unroll
      for (int a = 0; a < E::JL; ++a)
#pragma unroll
        for (int r = 0; r < E::RL; ++r) {
          int p, n;
          if (E::out_pos(a, r, p, n) && p < nvalid) fp[n * zstride + p] = o[a][r];
        }
    }
  }
}

// ---------------------------------------------------------------------------
// spectral update shared by zfwd and the kx = 0 fix-up
// ---------------------------------------------------------------------------
enum StageMode {
  SM_RHS = 0,                       // store the right-hand side
  SM_RK1 = 1, SM_RK2 = 2, SM_RK3 = 3, SM_RK4 = 4,   // IF-RK4 stages
  SM_AB2_EULER = 10, SM_AB2_MID = 11, SM_AB2 = 12,  // IF-AB2 passes
  SM_LAMB = 20,                     // store the raw transform (no update)
  // a stepper whose per-mode update runs in the z-forward epilogue; only
  // kernel instances with the mode as a compile-time constant carry it
  SM_AB2V = 30                      // variable-step IF-AB2 (sc_ab2v.cuh)
};

template <typename T> struct StageArgs {
  int mode;
  C2<T>* v[3];          // state v^_n (read)
  C2<T>* vout[3];       // where the final stage writes v^_{n+1} (normally == v)
  const C2<T>* sin[3];  // stage input (forcing reads it)
  C2<T>* sout[3];       // next stage input
  C2<T>* acc[3];        // RK accumulator / AB2 history
  C2<T>* w[3];          // right-hand side output (SM_RHS)
  const C2<T>* v0[3];   // AB2 midpoint restart: state at t = 0
  C2<T>* side;          // kx = 0 plane of w before symmetrize: [(iz*ny+iy)*3+c]
  const T* ex;          // exp(-nu kx^2 dt/2), exp(-nu ky^2 dt/2), exp(-nu kz^2 dt/2)
  const T* ey;
  const T* ez;
  T dt;
  int forced;
  double fkmax2, eps;
  const double* kf_partial;
  int kf_tiles;
  int kf_ptile;         // tile width of the zinv kernel that wrote kf_partial
  double kcut2;
  int mask_rhs;         // also truncate the RHS (mask = rhs_and_step)
  int symmetrize;       // apply symmetrize.f90:32-64 to w
  int project;          // apply projection.f90 to w
  // fused z kernel: slots (field indices of the slab map) of the fields the
  // update reads, prefetched into L2 once a tile's Lamb vector is in
  int pf_n;
  int pf_slot[6];
  // SM_AB2V
  int pass;             // 0, 1 or >= 2 (ab2v_point)
  C2<T>* hist[3];       // the previous right-hand side o
  C2<T>* vinit[3];      // the initial field (pass 0 writes it, pass 1 reads it)
  double nu;            // viscosity
  double dto;           // the previous step
  double wgt[3];        // the pass's weights s, ek, dl (ab2v_weights)
  // forcing with a coefficient computed on the device (force_rot.f90): when
  // fcoef is set, w += (*fcoef) sin on the band fband_lo2 <= k2 < fkmax2
  const double* fcoef;
  double fband_lo2;
};


// What the update of a mode reads at each point besides w.
__host__ __device__ constexpr bool mode_reads_v(int m) {
  return m == SM_RK1 || m == SM_RK2 || m == SM_RK3 || m == SM_AB2_EULER || m == SM_AB2 ||
         m == SM_AB2_MID || m == SM_AB2V;
}
__host__ __device__ constexpr bool mode_reads_acc(int m) {
  return m == SM_RK2 || m == SM_RK3 || m == SM_RK4 || m == SM_AB2;
}

// Projection, optional RHS mask and the mode's update at one point, with the
// state (v, or v0 for the AB2 midpoint pass) and accumulator values already
// loaded.  w is the right-hand side after forcing and symmetrize.  With
// `snext` given, RK stages 1-3 return the next stage input there instead of
// storing it to st.sout.  kcut_b = k2_lt(st.kcut2), computed once per
// kernel.  MODE >= 0: the update mode as a compile-time constant (st.mode
// otherwise).
template <typename T, int MODE = -1>
__device__ __forceinline__ void finish_point_pre(const StageArgs<T>& st, const Geom& g, long long idx,
                                                 int ix, int iy, int iz, int kcut_b, C2<T>* w, const C2<T>* vv,
                                                 const C2<T>* av, C2<T>* snext = nullptr) {
  using C = C2<T>;
  const int kyi = wavenum(iy, g.ny), kzi = wavenum(iz, g.nz);
  const int k2i = ix * ix + kyi * kyi + kzi * kzi;
  const T kx = (T)ix, ky = (T)kyi, kz = (T)kzi;
  if (st.project && k2i > 0) {
    // projection.f90:24-28: w -= k (k.w)/(k^2 + tiny)
    C t = cadd(cadd(cscale(w[0], kx), cscale(w[1], ky)), cscale(w[2], kz));
    t = cscale(t, T(1) / (T)k2i);
    w[0] = csub(w[0], cscale(t, kx));
    w[1] = csub(w[1], cscale(t, ky));
    w[2] = csub(w[2], cscale(t, kz));
  }
  const bool cut = k2i >= kcut_b && !(ix == 0 && iy == 0 && iz == 0);
  if (st.mask_rhs && cut) w[0] = w[1] = w[2] = czero<C>();
  if constexpr (MODE == SM_AB2V) {
    // spectral_dns.f90:220-290 at this mode (ab2v_point); v = 0 where cut and
    // at the mean mode
    const int pass = st.pass;
    Cx<T> v[3], wc[3], o[3], z[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v[c] = cx(vv[c].x, vv[c].y);
      wc[c] = cx(w[c].x, w[c].y);
      o[c] = z[c] = cx(T(0), T(0));
      if (pass >= 2) {
        const C q = st.hist[c][idx];
        o[c] = cx(q.x, q.y);
      } else if (pass == 1) {
        const C q = st.vinit[c][idx];
        z[c] = cx(q.x, q.y);
      }
    }
    ab2v_point<T>(pass, k2i, cut || k2i == 0, (T)st.nu, st.dt, (T)st.dto, (T)st.wgt[0], (T)st.wgt[1],
                  (T)st.wgt[2], v, wc, o, z);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      st.vout[c][idx] = mk<C>(v[c].re, v[c].im);
      if (pass != 1) st.hist[c][idx] = mk<C>(o[c].re, o[c].im);
      if (pass == 0) st.vinit[c][idx] = mk<C>(z[c].re, z[c].im);
    }
    return;
  }
  const int mode = MODE >= 0 ? MODE : st.mode;
  if (mode == SM_RHS || mode == SM_LAMB) {
#pragma unroll
    for (int c = 0; c < 3; ++c) st.w[c][idx] = w[c];
    return;
  }
  const T E = st.ex[ix] * st.ey[iy] * st.ez[iz];
  const T E2 = E * E;
  const T dt = st.dt, hdt = T(0.5) * st.dt;
  const bool zero_mean_cut = cut || (ix == 0 && iy == 0 && iz == 0);
  switch (mode) {
    case SM_RK1:  // acc = E^2 dt w1 ; s2 = E (v + dt w1/2)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        st.acc[c][idx] = cscale(w[c], E2 * dt);
        const C sn = cscale(cadd(vv[c], cscale(w[c], hdt)), E);
        if (snext) snext[c] = sn;
        else st.sout[c][idx] = sn;
      }
      break;
    case SM_RK2:  // acc += 2 E dt w2 ; s3 = E v + dt w2/2
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        st.acc[c][idx] = cadd(av[c], cscale(w[c], T(2) * E * dt));
        const C sn = cadd(cscale(vv[c], E), cscale(w[c], hdt));
        if (snext) snext[c] = sn;
        else st.sout[c][idx] = sn;
      }
      break;
    case SM_RK3:  // acc <- E^2 v + (acc + 2 E dt w3)/6 (stage 4 then needs no v) ; s4 = E^2 v + E dt w3
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        st.acc[c][idx] = cadd(cscale(vv[c], E2), cscale(cadd(av[c], cscale(w[c], T(2) * E * dt)), T(1) / T(6)));
        const C sn = cadd(cscale(vv[c], E2), cscale(w[c], E * dt));
        if (snext) snext[c] = sn;
        else st.sout[c][idx] = sn;
      }
      break;
    case SM_RK4:  // v = E^2 v + (acc + dt w4)/6 = acc' + dt w4/6 (acc' from stage 3), then the 2/3 mask
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        C vn = cadd(av[c], cscale(cscale(w[c], dt), T(1) / T(6)));
        if (cut) vn = czero<C>();
        if (snext) snext[c] = vn;
        else st.vout[c][idx] = vn;
      }
      break;
    case SM_AB2_EULER:  // v = (v + dt/2 w) sqrt(expk2) ; history = w
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        C vn = cscale(cadd(vv[c], cscale(w[c], hdt)), E);
        st.acc[c][idx] = w[c];
        st.vout[c][idx] = zero_mean_cut ? czero<C>() : vn;
      }
      break;
    case SM_AB2_MID:  // v = v0 expk2 + dt w sqrt(expk2)   (history kept)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        C vn = cadd(cscale(vv[c], E2), cscale(w[c], dt * E));
        st.vout[c][idx] = zero_mean_cut ? czero<C>() : vn;
      }
      break;
    case SM_AB2:  // v = (v + (3 w - expk2 o) dt/2) expk2 ; o = w
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        C d = csub(cscale(w[c], T(3)), cscale(av[c], E2));
        C vn = cscale(cadd(vv[c], cscale(d, hdt)), E2);
        st.acc[c][idx] = w[c];
        st.vout[c][idx] = zero_mean_cut ? czero<C>() : vn;
      }
      break;
    default:
      break;
  }
}

template <typename T, int MODE = -1>
__device__ __forceinline__ void load_state(const StageArgs<T>& st, long long idx, C2<T>* vv, C2<T>* av) {
  const int mode = MODE >= 0 ? MODE : st.mode;
  const bool rv = mode_reads_v(mode), ra = mode_reads_acc(mode);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (rv) vv[c] = mode == SM_AB2_MID ? st.v0[c][idx] : st.v[c][idx];
    if (ra) av[c] = st.acc[c][idx];
  }
}

template <typename T, int MODE = -1>
__device__ __forceinline__ void finish_point(const StageArgs<T>& st, const Geom& g, long long idx,
                                             int ix, int iy, int iz, int kcut_b, C2<T>* w) {
  C2<T> vv[3], av[3];
  load_state<T, MODE>(st, idx, vv, av);
  finish_point_pre<T, MODE>(st, g, idx, ix, iy, iz, kcut_b, w, vv, av);
}

// K_f of force.f90:16-22 from the zinv partial sums, fixed order.
// Visits exactly the (tile, ky) blocks that zinv wrote: (t*P)^2 + ky^2 < fkmax2.
__device__ __forceinline__ double forcing_energy(const double* partial, int tiles, int P, int ny,
                                                 double fkmax2) {
  double s = 0.0;
  for (int t = 0; t < tiles; ++t)
    for (int iy = 0; iy < ny; ++iy) {
      const double ky = wavenum(iy, ny), kx0 = (double)t * P;
      if (kx0 * kx0 + ky * ky < fkmax2) s += partial[(long long)t * ny + iy];
    }
  return s;
}

// ---------------------------------------------------------------------------
// zfwd: z-axis forward pass + spectral update.  NIN = 3 (Lamb vector) or 9
// (Lamb vector + tau_ij, order 11 12 13 22 23 33).
// ---------------------------------------------------------------------------
// w (the engine's output layout) += the z-transformed field f of the
// right-hand side: the Lamb vector (f < 3) or tau_ij (f >= 3, order 11 12 13
// 22 23 33: w_i -= i k_j tau_ij, spectral_les.f90:232-234).
template <typename E, typename T>
__device__ __forceinline__ void zfwd_accumulate(C2<T> (&w)[E::JL][E::RL][3], const C2<T> (&o)[E::JL][E::RL], int f,
                                                int kx0, T ky, const Geom& g) {
#pragma unroll
  for (int a = 0; a < E::JL; ++a)
#pragma unroll
    for (int r = 0; r < E::RL; ++r) {
      if (f < 3) {
#pragma unroll
        for (int c = 0; c < 3; ++c)
          if (c == f) w[a][r][c] = o[a][r];
      } else {
        int p, n;
        E::out_pos(a, r, p, n);
        const T kx = (T)(kx0 + p), kz = (T)wavenum(n, g.nz);
        const C2<T> t = o[a][r];
        switch (f - 3) {
          case 0: w[a][r][0] = csub(w[a][r][0], cmuli(cscale(t, kx))); break;
          case 1:
            w[a][r][0] = csub(w[a][r][0], cmuli(cscale(t, ky)));
            w[a][r][1] = csub(w[a][r][1], cmuli(cscale(t, kx)));
            break;
          case 2:
            w[a][r][0] = csub(w[a][r][0], cmuli(cscale(t, kz)));
            w[a][r][2] = csub(w[a][r][2], cmuli(cscale(t, kx)));
            break;
          case 3: w[a][r][1] = csub(w[a][r][1], cmuli(cscale(t, ky))); break;
          case 4:
            w[a][r][1] = csub(w[a][r][1], cmuli(cscale(t, kz)));
            w[a][r][2] = csub(w[a][r][2], cmuli(cscale(t, ky)));
            break;
          default: w[a][r][2] = csub(w[a][r][2], cmuli(cscale(t, kz))); break;
        }
      }
    }
}

// The z-forward pass's update of tile (kx0, iy) from w in the engine's
// output layout: the RHS itself (SM_LAMB), else forcing, symmetrize and the
// mode's update.  s_coef: a shared double of the block.
template <typename E, typename T>
__device__ __forceinline__ void zfwd_finish(C2<T> (&w)[E::JL][E::RL][3], const StageArgs<T>& st, const Geom& g,
                                            int kx0, int iy, int nvalid, long long base, long long zstride,
                                            double& s_coef) {
  using C = C2<T>;
  const T ky = (T)wavenum(iy, g.ny);
  if (st.mode == SM_LAMB) {
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        if (E::out_pos(a, r, p, n) && p < nvalid) {
          const long long idx = base + n * zstride + p;
#pragma unroll
          for (int c = 0; c < 3; ++c) st.w[c][idx] = w[a][r][c];
        }
      }
    return;
  }
  // forcing coefficient a = eps / (2 K_f) (force.f90:23)
  const bool fblock = st.forced && ((double)kx0 * kx0 + (double)ky * ky < st.fkmax2);
  const int kyi = wavenum(iy, g.ny), fk_b = k2_lt(st.fkmax2), kc_b = k2_lt(st.kcut2);
  if (fblock) {
    if (threadIdx.x == 0) {
      const double kf = forcing_energy(st.kf_partial, st.kf_tiles, st.kf_ptile, g.ny, st.fkmax2);
      s_coef = st.eps / (2.0 * kf);
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
      C* wp = w[a][r];
      if (fblock) {
        const int kz = wavenum(iz, g.nz);
        if (ix * ix + kyi * kyi + kz * kz < fk_b) {
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
          // copy targets are finished by the fix-up kernel
          if (iz > g.nz / 2 || (iz == 0 && iy > g.ny / 2)) continue;
        }
        if (iy == g.ny / 2 || iz == g.nz / 2 || ix == g.nxh - 1 || (ix == 0 && iy == 0 && iz == 0))
          wp[0] = wp[1] = wp[2] = czero<C>();
      }
      finish_point<T>(st, g, idx, ix, iy, iz, kc_b, wp);
    }
}

template <typename T, int LOGN, int NIN>
__global__ void __launch_bounds__(PencilCfg<T, LOGN>::NT, PencilCfg<T, LOGN>::MINB_FUSED)
zfwd_stage_kernel(FieldList<T> fin, StageArgs<T> st, Geom g, const C2<T>* __restrict__ tw) {
  using Cfg = PencilCfg<T, LOGN>;
  using E = typename Cfg::Engine;
  using C = C2<T>;
  constexpr int P = Cfg::P;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  __shared__ double s_coef;
  const int kx0 = blockIdx.x * P;
  const int iy = blockIdx.y;
  const int nvalid = min(P, g.nxh - kx0);
  const long long zstride = (long long)g.ny * g.nxp;
  const long long base = (long long)iy * g.nxp + kx0;
  const T ky = (T)wavenum(iy, g.ny);

  C w[E::JL][E::RL][3];
  for (int f = 0; f < NIN; ++f) {
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
    zfwd_accumulate<E, T>(w, o, f, kx0, ky, g);
  }
  zfwd_finish<E, T>(w, st, g, kx0, iy, nvalid, base, zstride, s_coef);
}

// Hermitian copy on the kx = 0 plane (symmetrize.f90:52-62):
// w(0,iy,iz) = conj(w(0,-iy,-iz)) for iz > nz/2, and for iz = 0, iy > ny/2.
template <typename T, int MODE = -1>
__global__ void fixup_kx0_kernel(StageArgs<T> st, Geom g) {
  using C = C2<T>;
  const long long total = (long long)g.ny * g.nz;
  const int kc_b = k2_lt(st.kcut2);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int iy = (int)(t % g.ny), iz = (int)(t / g.ny);
    if (!(iz > g.nz / 2 || (iz == 0 && iy > g.ny / 2))) continue;
    const int sy = (g.ny - iy) % g.ny, sz = (g.nz - iz) % g.nz;
    C w[3];
    const long long s = ((long long)sz * g.ny + sy) * 3;
#pragma unroll
    for (int c = 0; c < 3; ++c) w[c] = (iy == g.ny / 2) ? czero<C>() : cconj(st.side[s + c]);
    const long long idx = ((long long)iz * g.ny + iy) * g.nxp;
    finish_point<T, MODE>(st, g, idx, 0, iy, iz, kc_b, w);
  }
}

// ---------------------------------------------------------------------------
// xpass: per-row c2r, physical-space product, r2c
// ---------------------------------------------------------------------------
enum XpMode { XP_DNS = 0, XP_SMAG = 1, XP_C2R3 = 2, XP_R2C3 = 3, XP_ADJ = 4 };
// modes of the warp-per-row x-pass (sc_xwarp.cuh)
enum XwMode { XW_DNS = 0, XW_ADJ = 1, XW_SMAG = 2 };
template <int MODE> struct XpIO;
template <> struct XpIO<XP_DNS> { static constexpr int fin = 6, fout = 3; };
template <> struct XpIO<XP_SMAG> { static constexpr int fin = 12, fout = 9; };
template <> struct XpIO<XP_C2R3> { static constexpr int fin = 3, fout = 3; };
template <> struct XpIO<XP_R2C3> { static constexpr int fin = 3, fout = 3; };
template <> struct XpIO<XP_ADJ> { static constexpr int fin = 9, fout = 6; };   // (u, w, phi) -> (w x phi, phi x u)

template <typename T> struct XArgs {
  const C2<T>* twx;        // the twiddle table base (WarpTw blocks after entry 4096)
  int* err;                // device error word of the bounded waits (may be nullptr)
  T scale;                 // 1/(nx ny nz)
  const double* c1;        // device scalar: Smagorinsky c1 (or dynamic cs2)
  double delta2;           // filter width squared
  long long rows;          // ny*nz
};

template <typename T, int LOGM, int MODE> struct XpCfg {
  static constexpr int M = 1 << LOGM;
  static constexpr int FIN = XpIO<MODE>::fin, FOUT = XpIO<MODE>::fout;
  static constexpr int FMAX = FIN > FOUT ? FIN : FOUT;
  static constexpr int BUDGET = sizeof(T) == 4 ? 6144 : 3072;   // complex elems (48 KB)
  static constexpr int RB0 = BUDGET / (M * FMAX);
  static constexpr int RB = RB0 < 1 ? 1 : (RB0 > 64 ? 64 : RB0);
  static constexpr int PA = RB * FIN, PSA = PA | 1;
  static constexpr int PB = RB * FOUT, PSB = PB | 1;
  static constexpr int JOBS = (PA * M / 8) > 0 ? PA * M / 8 : 1;
  static constexpr int NT = JOBS >= 256 ? 256 : ((JOBS + 31) / 32) * 32;
  using EA = FFTEngine<T, LOGM, PA, PSA, NT, false, 3>;
  using EB = FFTEngine<T, LOGM, PB, PSB, NT, false, 3>;
  static constexpr int MP = EA::NPAD;   // padded point count (see FFTEngine::sidx)
  static constexpr int SMEM_ELEMS = (MP * PSA > MP * PSB ? MP * PSA : MP * PSB);
  static constexpr size_t SMEM = sizeof(C2<T>) * SMEM_ELEMS;
  static constexpr int MINB = SMEM * 3 <= 220 * 1024 ? 3 : 2;
};

template <typename T, int LOGM, int MODE>
__global__ void __launch_bounds__(XpCfg<T, LOGM, MODE>::NT, XpCfg<T, LOGM, MODE>::MINB)
xpass_kernel(FieldList<T> fin, FieldList<T> fout, Geom g, const C2<T>* __restrict__ twM,
             const C2<T>* __restrict__ twN, XArgs<T> xa) {
  using Cfg = XpCfg<T, LOGM, MODE>;
  using EA = typename Cfg::EA;
  using EB = typename Cfg::EB;
  using C = C2<T>;
  constexpr int M = Cfg::M, RB = Cfg::RB, NT = Cfg::NT;
  constexpr int PSA = Cfg::PSA, PSB = Cfg::PSB, PB = Cfg::PB;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  const long long row0 = (long long)blockIdx.x * RB;
  const long long pitch = g.nxp;

  C inB[EB::J1][EB::R1];
  if constexpr (MODE != XP_R2C3) {
    // ---- phase A: half-complex rows -> packed physical rows (c2r) ----
    C inA[EA::J1][EA::R1], outA[EA::JL][EA::RL];
#pragma unroll
    for (int a = 0; a < EA::J1; ++a)
#pragma unroll
      for (int r = 0; r < EA::R1; ++r) {
        int p, k;
        bool ok = EA::in_pos(a, r, p, k);
        const int f = p / RB, rl = p % RB;
        const long long row = row0 + rl;
        C z = czero<C>();
        if (ok && row < xa.rows) {
          const C* __restrict__ rp = fin.f[f] + row * pitch;
          C xk = rp[k], xm = rp[M - k];
          if (k == 0) { xk.y = 0; xm.y = 0; }   // DC and Nyquist are real
          const C e = cadd(xk, cconj(xm));
          const C o = cmulc(csub(xk, cconj(xm)), __ldg(&twN[k]));   // * e^{+2 pi i k/N}
          z = cadd(e, cmuli(o));
        }
        inA[a][r] = z;
      }
    EA::template run<true>(inA, outA, sm, twM);
    if constexpr (MODE == XP_C2R3) {
#pragma unroll
      for (int a = 0; a < EA::JL; ++a)
#pragma unroll
        for (int r = 0; r < EA::RL; ++r) {
          int p, m;
          bool ok = EA::out_pos(a, r, p, m);
          const int f = p / RB, rl = p % RB;
          const long long row = row0 + rl;
          if (ok && row < xa.rows) fout.f[f][row * pitch + m] = outA[a][r];
        }
      return;
    }
#pragma unroll
    for (int a = 0; a < EA::JL; ++a)
#pragma unroll
      for (int r = 0; r < EA::RL; ++r) {
        int p, m;
        if (EA::out_pos(a, r, p, m)) sm[EA::sidx(m) * PSA + p] = outA[a][r];
      }
    __syncthreads();
    // ---- physical-space products ----
    const T sc = xa.scale;
    T tcoef = T(0);
    if constexpr (MODE == XP_SMAG) tcoef = (T)(-2.0 * (*xa.c1) * xa.delta2) * sc;
#pragma unroll
    for (int a = 0; a < EB::J1; ++a)
#pragma unroll
      for (int r = 0; r < EB::R1; ++r) {
        int p, m;
        bool ok = EB::in_pos(a, r, p, m);
        C res = czero<C>();
        if (ok) {
          const int gq = p / RB, rl = p % RB;
          const C* row = sm + EA::sidx(m) * PSA + rl;
          auto U = [&](int c) { return row[c * RB]; };
          if (MODE == XP_ADJ) {
            // adjoint of the Lamb product: a_u = w x phi, a_w = phi x u
            const int c1 = (gq + 1) % 3, c2 = (gq + 2) % 3;
            const int A = gq < 3 ? 3 : 6, B = gq < 3 ? 6 : 0;
            const C pa = U(A + c1), pb = U(A + c2), qa = U(B + c1), qb = U(B + c2);
            res = mk<C>(pa.x * qb.x - pb.x * qa.x, pa.y * qb.y - pb.y * qa.y);
          } else if (gq < 3) {
            // convec_dns.f90:30-42: Lamb vector u x w on even (re) / odd (im) points
            const int c1 = (gq + 1) % 3, c2 = (gq + 2) % 3;
            const C ua = U(c1), ub = U(c2), wa = U(3 + c1), wb = U(3 + c2);
            res = mk<C>((ua.x * wb.x - ub.x * wa.x) * sc, (ua.y * wb.y - ub.y * wa.y) * sc);
          } else {
            // smag.f90:41-64: tau_ij = -2 c1 D^2 |S| S_ij / N^3
            const C s11 = U(6), s12 = U(7), s13 = U(8), s22 = U(9), s23 = U(10), s33 = U(11);
            const T sr = sqrt(T(2) * (s11.x * s11.x + s22.x * s22.x + s33.x * s33.x +
                                      T(2) * (s12.x * s12.x + s13.x * s13.x + s23.x * s23.x)));
            const T si = sqrt(T(2) * (s11.y * s11.y + s22.y * s22.y + s33.y * s33.y +
                                      T(2) * (s12.y * s12.y + s13.y * s13.y + s23.y * s23.y)));
            const C sij = U(6 + gq - 3);
            res = mk<C>(sr * sij.x * tcoef, si * sij.y * tcoef);
          }
        }
        inB[a][r] = res;
      }
    __syncthreads();
  } else {
#pragma unroll
    for (int a = 0; a < EB::J1; ++a)
#pragma unroll
      for (int r = 0; r < EB::R1; ++r) {
        int p, m;
        bool ok = EB::in_pos(a, r, p, m);
        const int gq = p / RB, rl = p % RB;
        const long long row = row0 + rl;
        inB[a][r] = (ok && row < xa.rows) ? fin.f[gq][row * pitch + m] : czero<C>();
      }
  }
  if constexpr (MODE != XP_C2R3) {
    // ---- phase B: packed physical rows -> half-complex rows (r2c) ----
    C outB[EB::JL][EB::RL];
    EB::template run<false>(inB, outB, sm, twM);
#pragma unroll
    for (int a = 0; a < EB::JL; ++a)
#pragma unroll
      for (int r = 0; r < EB::RL; ++r) {
        int p, m;
        if (EB::out_pos(a, r, p, m)) sm[EB::sidx(m) * PSB + p] = outB[a][r];
      }
    __syncthreads();
    constexpr int TOT = PB * (M + 1);
    for (int job = threadIdx.x; job < TOT; job += NT) {
      const int k = job % (M + 1), p = job / (M + 1);
      const int gq = p / RB, rl = p % RB;
      const long long row = row0 + rl;
      if (row >= xa.rows) continue;
      const C zk = sm[EB::sidx(k % M) * PSB + p];
      const C zm = cconj(sm[EB::sidx((M - k) % M) * PSB + p]);
      const C e = cadd(zk, zm);
      const C d = cmul(csub(zk, zm), __ldg(&twN[k]));      // * e^{-2 pi i k/N}
      const C x = cscale(csub(e, cmuli(d)), T(0.5));
      fout.f[gq][row * pitch + k] = x;
    }
  }
}

}  // namespace sc
