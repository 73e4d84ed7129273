// Batched 2D vorticity ensembles: members of mixed size N advance together,
// one persistent (cooperative) launch per RK stage.
//
// Physics per member (restated from the 2D solvers of the reference:
// spectral_dns_2d.f90:94,160-188 and turb_2d.f90:288-403):
//   u^ = i ky w^/k^2, v^ = -i kx w^/k^2,
//   N^ = -(i kx (u w)^ + i ky (v w)^), then symmetrize2d (symmetrize.f90:8-30)
//   and the 2/3 mask; integrating factor E = exp(-(alpha + nu8 k^8) dt/2)
//   in the division-free IF-RK4 (dns-deform.f90:160-230 rewritten).
// Layout per member: (N, nxp) complex rows (ky, kx), kx fastest, nxp >= N/2+1.
//
// One stage = three phases separated by a grid barrier:
//   P1 y-inverse: per kx-tile, generate u^, v^, w^ from the stage input and
//                 transform along ky (3 work fields);
//   P2 x-pass   : warp per row, c2r of u, v, w, products u w / N^2, v w / N^2,
//                 r2c (into work fields 0, 1);
//   P3 y-forward: transform the two products, form N^, symmetrize (the kx = 0
//                 conjugate pairs lie in one pencil: exchanged in shared
//                 memory), mask, and apply the RK stage.
// The grid barrier is a counter/generation pair with a bounded wait; a wait
// that gives up records an error and the launch returns.
#pragma once
#include "sc_xwarp.cuh"

namespace sc {

template <typename T> struct EnsMember {
  int n, logn, nxh, nxp, ptile, ntx;
  long long field;         // elements per field
  C2<T>* w;                // state
  C2<T>* s;                // stage input
  C2<T>* acc;              // RK accumulator
  C2<T>* work;             // 3 work fields
  T dt, alpha, nu8, scale; // scale = 1/N^2
  int item_y0, item_x0;    // first item of this member in the y phases / x phase
};

template <typename T> struct EnsArgs {
  const EnsMember<T>* m;
  int nm;
  int items_y, items_x;    // totals over members
  int stage;               // 1..4
  const C2<T>* tw;         // twiddles: table of length L at offset L
  unsigned* bar;           // [0] arrivals, [1] generation
  int* err;
};

// Launch shape of the stage kernel, the autotuner's search space: threads
// per CTA, CTAs per SM (the register budget), points per y-phase tile
// (tile width P = YPTS / N pencils, at most 16) and the FFT's largest radix.
// OUTLINE: the phase functions are called out of line, each allocated its
// own registers, and the y-forward accumulator sits in shared memory (fewer
// spills, but call overhead); otherwise everything is inlined.
template <int NT_, int MINB_, int YPTS_, int RMAX_, bool OUTLINE_> struct EnsShape {
  static constexpr int NT = NT_, MINB = MINB_, YPTS = YPTS_, RMAX = RMAX_;
  static constexpr bool OUTLINE = OUTLINE_;
  static constexpr int WARPS = NT_ / 32;
  static constexpr int ptile(int n) { return YPTS_ / n > 16 ? 16 : (YPTS_ / n < 1 ? 1 : YPTS_ / n); }
  // dynamic shared memory (complex elements): a y tile and the y-forward
  // accumulator slots, or per warp the x-pass transpose buffer and w row of
  // the largest row length
  static constexpr int smem_elems() {
    return (OUTLINE_ ? 2 : 1) * YPTS_ > WARPS * (544 + 512) ? (OUTLINE_ ? 2 : 1) * YPTS_ : WARPS * (544 + 512);
  }
};

template <typename T, class SH, int LOGN> struct EnsY {
  static constexpr int N = 1 << LOGN;
  static constexpr int P = SH::ptile(N);
  using E = FFTEngine<T, LOGN, P, P, SH::NT, true, 0, false, SH::RMAX>;
};

// Bounded grid-wide barrier for a cooperative launch.
__device__ __forceinline__ bool ens_grid_sync(unsigned* bar, int* err) {
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = bar + 1;
    const unsigned gen = *vgen;
    __threadfence();
    const unsigned arrived = atomicAdd(bar, 1u);
    ok = 1;
    if (arrived == gridDim.x - 1) {
      bar[0] = 0;
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long it = 0;
      while (*vgen == gen) {
        if (++it > (1LL << 24)) {   // ~1 s of 64 ns sleeps
          atomicExch(err, 4);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

template <typename T>
__device__ __forceinline__ int ens_member_of(const EnsArgs<T>& ea, int item, bool xphase) {
  int lo = 0;
  for (int i = 1; i < ea.nm; ++i) {
    const int s = xphase ? ea.m[i].item_x0 : ea.m[i].item_y0;
    if (item >= s) lo = i;
  }
  return lo;
}

// P1: y-inverse of u^, v^, w^ generated from the stage input
template <typename T, class SH, int LOGN>
__device__ __forceinline__ void ens_yinv(const EnsMember<T>& mb, int tile, C2<T>* sm, const C2<T>* __restrict__ tw) {
  using Y = EnsY<T, SH, LOGN>;
  using E = typename Y::E;
  using C = C2<T>;
  constexpr int P = Y::P;
  const int kx0 = tile * P;
  const int nvalid = min(P, mb.nxh - kx0);
  for (int f = 0; f < 3; ++f) {
    C in[E::J1][E::R1], o[E::JL][E::RL];
#pragma unroll
    for (int a = 0; a < E::J1; ++a)
#pragma unroll
      for (int r = 0; r < E::R1; ++r) {
        int p, n;
        const bool ok = E::in_pos(a, r, p, n) && p < nvalid;
        const T kx = (T)(kx0 + p), ky = (T)wavenum(n, mb.n);
        const T k2 = kx * kx + ky * ky;
        const T ik2 = k2 > T(0) ? T(1) / k2 : T(0);
        const C x = ok ? mb.s[(long long)n * mb.nxp + kx0 + p] : czero<C>();
        in[a][r] = f == 0 ? cmuli(cscale(x, ky * ik2)) : (f == 1 ? cmulmi(cscale(x, kx * ik2)) : x);
      }
    E::template run<true>(in, o, sm, tw + Y::N);
    C* __restrict__ fp = mb.work + f * mb.field + kx0;
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        if (E::out_pos(a, r, p, n) && p < nvalid) fp[(long long)n * mb.nxp + p] = o[a][r];
      }
  }
}

// P2: one warp per row: c2r of u, v, w; products; r2c into work fields 0, 1
template <typename T, int LOGM>
__device__ __forceinline__ void ens_xrow(const EnsMember<T>& mb, int row, C2<T>* smw, const C2<T>* __restrict__ tw) {
  using WF = WarpFFT<T, LOGM>;
  using C = C2<T>;
  constexpr int M = WF::M, E = WF::E;
  const int lane = threadIdx.x & 31;
  const C* __restrict__ twM = tw + M;
  const C* __restrict__ twN = tw + 2 * M;
  // twiddles from the lane-major tables after the power-of-two lengths
  constexpr bool TX = WarpTw::covers(LOGM);
  const C* __restrict__ tx = TX ? tw + WarpTw::offset(LOGM) : nullptr;
  const long long off = (long long)row * mb.nxp;
  auto load_z = [&](int f, C (&x)[E]) {
    const C* __restrict__ rp = mb.work + f * mb.field + off;
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int k = lane + 32 * r;
      C xk = rp[k], xm = rp[M - k];
      if (k == 0) { xk.y = 0; xm.y = 0; }
      const C e = cadd(xk, cconj(xm));
      const C o = cmulc(csub(xk, cconj(xm)), __ldg(&twN[k]));
      x[r] = cadd(e, cmuli(o));
    }
  };
  C a[E];
  C* wsm = smw + WF::SMEM;   // w (scrambled order) at [i * 32 + lane]
  load_z(2, a);
  WF::template nat_to_scr<true, TX>(a, smw, twM, lane, tx);
#pragma unroll
  for (int i = 0; i < E; ++i) wsm[i * 32 + lane] = a[i];
  const T sc = mb.scale;
  for (int f = 0; f < 2; ++f) {
    load_z(f, a);
    WF::template nat_to_scr<true, TX>(a, smw, twM, lane, tx);
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const C wv = wsm[i * 32 + lane];
      a[i] = mk<C>(a[i].x * wv.x * sc, a[i].y * wv.y * sc);
    }
    WF::template scr_to_nat<false, TX>(a, smw, twM, lane, tx);
    C* __restrict__ op = mb.work + f * mb.field + off;
    const int src = (32 - lane) & 31;
#pragma unroll
    for (int r = 0; r < E; ++r) {
      C zm;
      zm.x = __shfl_sync(0xffffffffu, a[E - 1 - r].x, src);
      zm.y = __shfl_sync(0xffffffffu, a[E - 1 - r].y, src);
      if (lane == 0) zm = a[(E - r) % E];
      const int k = lane + 32 * r;
      const C zmc = cconj(zm);
      const C e = cadd(a[r], zmc);
      const C d = cmul(csub(a[r], zmc), __ldg(&twN[k]));
      op[k] = cscale(csub(e, cmuli(d)), T(0.5));
      if (k == 0) {
        const C d0 = cmul(csub(a[r], zmc), __ldg(&twN[M]));
        op[M] = cscale(csub(e, cmuli(d0)), T(0.5));
      }
    }
  }
}

// P3: y-forward of the products, N^, symmetrize2d, mask, RK stage.  With
// SH::OUTLINE the first product's contribution waits in thread-private
// shared-memory slots above the tile (sm[YPTS ...]) instead of registers.
template <typename T, class SH, int LOGN>
__device__ __forceinline__ void ens_yfwd(const EnsMember<T>& mb, int tile, int stage, C2<T>* sm,
                                      const C2<T>* __restrict__ tw) {
  using Y = EnsY<T, SH, LOGN>;
  using E = typename Y::E;
  using C = C2<T>;
  constexpr int P = Y::P, N = Y::N;
  const int kx0 = tile * P;
  const int nvalid = min(P, mb.nxh - kx0);
  C* nlbuf = sm + SH::YPTS;
  C nl[E::JL][E::RL], nl0[E::JL][E::RL];
  for (int f = 0; f < 2; ++f) {
    C in[E::J1][E::R1], o[E::JL][E::RL];
#pragma unroll
    for (int a = 0; a < E::J1; ++a)
#pragma unroll
      for (int r = 0; r < E::R1; ++r) {
        int p, n;
        bool ok = E::in_pos(a, r, p, n) && p < nvalid;
        in[a][r] = ok ? mb.work[f * mb.field + (long long)n * mb.nxp + kx0 + p] : czero<C>();
      }
    E::template run<false>(in, o, sm, tw + N);
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        E::out_pos(a, r, p, n);
        const T k = f == 0 ? (T)(kx0 + p) : (T)wavenum(n, N);
        const C t = cmulmi(cscale(o[a][r], k));   // -i k X
        if constexpr (SH::OUTLINE) {
          C* slot = nlbuf + (a * E::RL + r) * SH::NT + threadIdx.x;
          if (f == 0) *slot = t;
          else nl[a][r] = cadd(*slot, t);
        } else {
          if (f == 0) nl0[a][r] = t;
          else nl[a][r] = cadd(nl0[a][r], t);
        }
      }
  }
  // symmetrize2d: zero ky = -N/2, kx = N/2 and the mean; kx = 0 copies
  const double kc = 2.0 * (N / 2) / 3.0;
  const int kc_b = k2_lt(kc * kc);
  if (kx0 == 0) {
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        if (E::out_pos(a, r, p, n) && p == 0) sm[n] = (n == N / 2 || n == 0) ? czero<C>() : nl[a][r];
      }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < E::JL; ++a)
#pragma unroll
      for (int r = 0; r < E::RL; ++r) {
        int p, n;
        if (E::out_pos(a, r, p, n) && p == 0 && n > N / 2) nl[a][r] = cconj(sm[N - n]);
      }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < E::JL; ++a)
#pragma unroll
    for (int r = 0; r < E::RL; ++r) {
      int p, n;
      if (!(E::out_pos(a, r, p, n) && p < nvalid)) continue;
      const int ix = kx0 + p;
      const int ky = wavenum(n, N);
      const int k2i = ix * ix + ky * ky;
      C w = nl[a][r];
      if (n == N / 2 || ix == mb.nxh - 1 || (ix == 0 && n == 0) || k2i >= kc_b) w = czero<C>();
      const T k2 = (T)k2i, k4 = k2 * k2;   // exact: k2 < 2^24
      const T arg = (mb.alpha + mb.nu8 * (k4 * k4)) * mb.dt * T(0.5);
      const T Ef = exp(-arg);
      const T E2 = Ef * Ef, dt = mb.dt, hdt = T(0.5) * mb.dt;
      const long long idx = (long long)n * mb.nxp + ix;
      // stage 3 leaves E^2 v + (acc + 2 E dt w3)/6 in acc, so stage 4 reads no v
      const C v = stage < 4 ? mb.w[idx] : czero<C>();
      switch (stage) {
        case 1:
          mb.acc[idx] = cscale(w, E2 * dt);
          mb.s[idx] = cscale(cadd(v, cscale(w, hdt)), Ef);
          break;
        case 2:
          mb.acc[idx] = cadd(mb.acc[idx], cscale(w, T(2) * Ef * dt));
          mb.s[idx] = cadd(cscale(v, Ef), cscale(w, hdt));
          break;
        case 3:
          mb.acc[idx] = cadd(cscale(v, E2), cscale(cadd(mb.acc[idx], cscale(w, T(2) * Ef * dt)), T(1) / T(6)));
          mb.s[idx] = cadd(cscale(v, E2), cscale(w, Ef * dt));
          break;
        default:   // v = E^2 v + (acc + dt w4)/6 = acc' + dt w4/6
          mb.w[idx] = cadd(mb.acc[idx], cscale(cscale(w, dt), T(1) / T(6)));
          break;
      }
    }
}

// Out-of-line entry points of the phases (SH::OUTLINE).
template <typename T, class SH, int LOGN>
__device__ __noinline__ void ens_yinv_call(const EnsMember<T>& mb, int tile, C2<T>* sm, const C2<T>* tw) {
  ens_yinv<T, SH, LOGN>(mb, tile, sm, tw);
}
template <typename T, int LOGM>
__device__ __noinline__ void ens_xrow_call(const EnsMember<T>& mb, int row, C2<T>* smw, const C2<T>* tw) {
  ens_xrow<T, LOGM>(mb, row, smw, tw);
}
template <typename T, class SH, int LOGN>
__device__ __noinline__ void ens_yfwd_call(const EnsMember<T>& mb, int tile, int stage, C2<T>* sm,
                                           const C2<T>* tw) {
  ens_yfwd<T, SH, LOGN>(mb, tile, stage, sm, tw);
}
template <typename T, class SH, int LOGN>
__device__ __forceinline__ void ens_p1(const EnsMember<T>& mb, int t, C2<T>* sm, const C2<T>* tw) {
  if constexpr (SH::OUTLINE) ens_yinv_call<T, SH, LOGN>(mb, t, sm, tw);
  else ens_yinv<T, SH, LOGN>(mb, t, sm, tw);
}
template <typename T, class SH, int LOGM>
__device__ __forceinline__ void ens_p2(const EnsMember<T>& mb, int row, C2<T>* smw, const C2<T>* tw) {
  if constexpr (SH::OUTLINE) ens_xrow_call<T, LOGM>(mb, row, smw, tw);
  else ens_xrow<T, LOGM>(mb, row, smw, tw);
}
template <typename T, class SH, int LOGN>
__device__ __forceinline__ void ens_p3(const EnsMember<T>& mb, int t, int stage, C2<T>* sm, const C2<T>* tw) {
  if constexpr (SH::OUTLINE) ens_yfwd_call<T, SH, LOGN>(mb, t, stage, sm, tw);
  else ens_yfwd<T, SH, LOGN>(mb, t, stage, sm, tw);
}

// One RK stage for every member.  Stage 1 reads the state as its input.
template <typename T, class SH>
__global__ void __launch_bounds__(SH::NT, SH::MINB) ens_stage_kernel(EnsArgs<T> ea) {
  using C = C2<T>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C* sm = reinterpret_cast<C*>(smraw);
  // P1
  for (int item = blockIdx.x; item < ea.items_y; item += gridDim.x) {
    const int mi = ens_member_of(ea, item, false);
    EnsMember<T> mb = ea.m[mi];
    if (ea.stage == 1) mb.s = mb.w;
    const int t = item - mb.item_y0;
    switch (mb.logn) {
      case 6: ens_p1<T, SH, 6>(mb, t, sm, ea.tw); break;
      case 7: ens_p1<T, SH, 7>(mb, t, sm, ea.tw); break;
      case 8: ens_p1<T, SH, 8>(mb, t, sm, ea.tw); break;
      case 9: ens_p1<T, SH, 9>(mb, t, sm, ea.tw); break;
      default: ens_p1<T, SH, 10>(mb, t, sm, ea.tw); break;
    }
  }
  if (!ens_grid_sync(ea.bar, ea.err)) return;
  // P2: SH::WARPS rows per item
  {
    const int warp = threadIdx.x >> 5;
    for (int item = blockIdx.x; item < ea.items_x; item += gridDim.x) {
      const int mi = ens_member_of(ea, item, true);
      const EnsMember<T>& mb = ea.m[mi];
      const int row = (item - mb.item_x0) * SH::WARPS + warp;
      if (row >= mb.n) continue;
      C* smw = sm + warp * (WarpFFT<T, 9>::SMEM + 512);   // transpose buffer + w row, largest size
      const C* tw = ea.tw;   // WarpFFT needs the tables of M and N = 2M at tw + M, tw + 2M
      switch (mb.logn - 1) {
        case 5: ens_p2<T, SH, 5>(mb, row, smw, tw); break;
        case 6: ens_p2<T, SH, 6>(mb, row, smw, tw); break;
        case 7: ens_p2<T, SH, 7>(mb, row, smw, tw); break;
        case 8: ens_p2<T, SH, 8>(mb, row, smw, tw); break;
        default: ens_p2<T, SH, 9>(mb, row, smw, tw); break;
      }
    }
  }
  if (!ens_grid_sync(ea.bar, ea.err)) return;
  // P3
  for (int item = blockIdx.x; item < ea.items_y; item += gridDim.x) {
    const int mi = ens_member_of(ea, item, false);
    EnsMember<T> mb = ea.m[mi];
    const int t = item - mb.item_y0;
    switch (mb.logn) {
      case 6: ens_p3<T, SH, 6>(mb, t, ea.stage, sm, ea.tw); break;
      case 7: ens_p3<T, SH, 7>(mb, t, ea.stage, sm, ea.tw); break;
      case 8: ens_p3<T, SH, 8>(mb, t, ea.stage, sm, ea.tw); break;
      case 9: ens_p3<T, SH, 9>(mb, t, ea.stage, sm, ea.tw); break;
      default: ens_p3<T, SH, 10>(mb, t, ea.stage, sm, ea.tw); break;
    }
    __syncthreads();
  }
}

// The compiled shapes (sc_ens_k_*.cu, one translation unit each), by variant
// number, <threads, CTAs per SM, tile points, radix, out of line>.  FP32:
// 0 <256, 2, 4096, 8, no>, 1 <256, 2, 4096, 8, yes>, 2 <512, 1, 8192, 8, no>,
// 3 <512, 1, 8192, 8, yes>, 4 <256, 2, 4096, 4, no>, 5 <512, 1, 4096, 8, no>.
// FP64: 0 <256, 2, 4096, 8, no>, 1 <256, 2, 4096, 8, yes>.

// A compiled variant as the host sees it.
struct EnsVariant {
  const void* kernel;   // ens_stage_kernel<T, Shape>
  int nt, minb, ypts, rmax, outline, smem_elems;
};

template <class SH, typename T> EnsVariant ens_variant_of() {
  return EnsVariant{reinterpret_cast<const void*>(&ens_stage_kernel<T, SH>), SH::NT, SH::MINB, SH::YPTS, SH::RMAX,
                    SH::OUTLINE ? 1 : 0, SH::smem_elems()};
}

// defined in sc_ens_variants.cu
EnsVariant ens_variant_f32(int v);
EnsVariant ens_variant_f64(int v);
constexpr int kEnsVariantsF32 = 6;
constexpr int kEnsVariantsF64 = 2;

}  // namespace sc
