// Warp-per-row x-axis pass of the right-hand side (c2r, Lamb vector, r2c).
//
// One warp owns one grid row (y, z): it transforms all six input fields of
// the row and the three outputs without any block-wide barrier.  An M-point
// FFT (M = nx/2 complex points, M = E * 32) runs as
//   radix-E DFT in registers over the 32-strided points of each lane,
//   twiddles W_M^{lane k1},
//   transpose through a padded warp-private shared buffer,
//   radix-E DFT in registers, twiddles W_32^{q u},
//   (32/E)-point DFT across each group of 32/E lanes: radix-2 warp-shuffle
//   butterflies down to groups of min(E, 32/E) lanes, then an all-to-all
//   shuffle exchange of register blocks inside each group and the rest of
//   the DFT in registers.
// The inverse (natural in, digit-scrambled out) leaves every field in the
// same scrambled order, so the Lamb product u x w is formed in registers; the
// forward transform is the transposed network (scrambled in, natural out).
//
// The c2r/r2c of the reference's packed rows (convec_dns.f90:22-47) use the
// half-length trick: z_m = x_{2m} + i x_{2m+1} is the M-point inverse of
// Z_k = (X_k + conj X_{M-k}) + i (X_k - conj X_{M-k}) e^{+2 pi i k/N}, and
// X_k = ((Z_k + conj Z_{M-k}) - i e^{-2 pi i k/N} (Z_k - conj Z_{M-k}))/2.
#pragma once
#include <utility>

#include "sc_launch.h"
#include "sc_passes.cuh"
#include "sc_tma.cuh"
#include "sc_tmem.cuh"

namespace sc {

template <int E, bool INV, typename C> __device__ __forceinline__ void dftE(C* v) {
  if constexpr (E == 2) dft2<INV>(v);
  else if constexpr (E == 4) dft4<INV>(v);
  else if constexpr (E == 8) dft8<INV>(v);
  else if constexpr (E == 16) dft16<INV>(v);
}

// cos and sin of 2 pi j / n at compile time, for the constant twiddles of
// the half-length c2r / r2c: quadrant and octant reduction to |x| <= pi/4,
// then the Maclaurin series of sin and cos (14 terms: far below double
// rounding on that interval).
namespace roots {
constexpr double kPi = 3.14159265358979323846264338327950288;
__host__ __device__ constexpr double mac_sin(double x) {
  double t = x, s = x;
  for (int k = 1; k < 14; ++k) { t *= -x * x / ((2.0 * k) * (2.0 * k + 1)); s += t; }
  return s;
}
__host__ __device__ constexpr double mac_cos(double x) {
  double t = 1, s = 1;
  for (int k = 1; k < 14; ++k) { t *= -x * x / ((2.0 * k - 1) * (2.0 * k)); s += t; }
  return s;
}
// n a multiple of 8; j in [0, n)
__host__ __device__ constexpr double cos2pi(int j, int n, bool want_sin) {
  const int quad = (4 * j) / n, jr = j - quad * (n / 4);          // angle = quad pi/2 + 2 pi jr/n
  const bool hi = 8 * jr > n;                                     // past pi/4: use the complement
  const double x = 2 * kPi * (hi ? n / 4 - jr : jr) / n;
  const double c0 = hi ? mac_sin(x) : mac_cos(x), s0 = hi ? mac_cos(x) : mac_sin(x);
  const double c = quad == 0 ? c0 : quad == 1 ? -s0 : quad == 2 ? -c0 : s0;
  const double s = quad == 0 ? s0 : quad == 1 ? c0 : quad == 2 ? -s0 : -c0;
  return want_sin ? s : c;
}
template <typename C, int N, int J> __device__ __forceinline__ C w_root() {   // W_N^J = e^{-2 pi i J/N}
  constexpr double c = cos2pi(J, N, false), s = cos2pi(J, N, true);
  return mk<C>(decltype(C::x)(c), decltype(C::x)(-s));
}
template <typename C, int N, int... J> __device__ __forceinline__ void fill(C* w, std::integer_sequence<int, J...>) {
  ((w[J] = w_root<C, N, J>()), ...);
}
}  // namespace roots

template <typename T, int LOGM> struct WarpFFT {
  using C = C2<T>;
  static constexpr int M = 1 << LOGM;
  static constexpr int E = M / 32;          // points per lane
  static constexpr int Q = 32 / E;          // lanes per row of the second level
  // The Q-point DFT across each group of Q lanes: radix-2 shuffle
  // butterflies on the lane bits h >= Q2 = min(Q, E), then an all-to-all
  // exchange of (E/Q2)-register blocks inside each group of Q2 lanes and a
  // Q2-point DFT in registers.
  static constexpr int Q2 = Q < E ? Q : E;
  static constexpr bool XCH = Q2 > 1;
  static constexpr int B = E / Q2;
  static constexpr int HMIN = XCH ? Q2 : 1;   // smallest butterfly lane bit
  static constexpr int ROW = 32 + Q;        // padded shared row: conflict-free transpose
  static constexpr int SMEM = E * ROW;      // complex elements per warp

  __device__ static __forceinline__ C twid(const C* __restrict__ tw, int m, bool inv) {
    const C w = __ldg(&tw[m]);
    return inv ? cconj(w) : w;
  }

  // x[j] *= w^j, j = 1 .. E-1, with w = tw[m] (conjugated for INV): one
  // table load per power (measured faster than forming the powers by
  // squarings and products from one load, SC_XW_TWPOW)
  template <bool INV>
  __device__ static __forceinline__ void twiddle_powers(C (&x)[E], const C* __restrict__ tw, int m) {
    if constexpr (E > 1) {
#ifndef SC_XW_TWPOW
#pragma unroll
      for (int j = 1; j < E; ++j) x[j] = cmul(x[j], twid(tw, m * j, INV));
#else
      C w[E];
      w[1] = twid(tw, m, INV);
#pragma unroll
      for (int j = 2; j < E; ++j) {
        const int hb = 1 << (31 - __clz(j));
        w[j] = hb == j ? mk<C>(w[j / 2].x * w[j / 2].x - w[j / 2].y * w[j / 2].y, T(2) * w[j / 2].x * w[j / 2].y)
                       : cmul(w[hb], w[j - hb]);
      }
#pragma unroll
      for (int j = 1; j < E; ++j) x[j] = cmul(x[j], w[j]);
#endif
    }
  }

  // The same products from the lane-major tables of WarpTw (tx): x[j] *=
  // W_M^{j lane} (first) or W_M^{j q E} (second level), one contiguous
  // warp-wide load per power where the M-point table's entries lane j lie
  // 8 j bytes apart.
  template <bool INV>
  __device__ static __forceinline__ void twiddle_first(C (&x)[E], const C* __restrict__ tx, int lane) {
#pragma unroll
    for (int j = 1; j < E; ++j) x[j] = cmul(x[j], twid(tx, (j - 1) * 32 + lane, INV));
  }
  template <bool INV>
  __device__ static __forceinline__ void twiddle_second(C (&x)[E], const C* __restrict__ tx, int q) {
#pragma unroll
    for (int j = 1; j < E; ++j) x[j] = cmul(x[j], twid(tx, (E - 1) * 32 + (j - 1) * Q + q, INV));
  }

  // all-to-all inside each group of Q2 lanes: afterwards lane q holds at
  // block p (registers p B .. p B + B-1) what lane p held at block q (q, p
  // the lane's index in its group).  One stage per lane bit h: the lane with
  // bit h clear keeps its blocks with bit h clear and trades the others with
  // lane q ^ h.  An involution.
  __device__ static __forceinline__ void exchange(C (&x)[E], int q) {
#pragma unroll
    for (int h = Q2 / 2; h >= 1; h >>= 1) {
      const bool up = (q & h) != 0;
#pragma unroll
      for (int b = 0; b < Q2; ++b) {
        if (b & h) continue;
#pragma unroll
        for (int i = 0; i < B; ++i) {
          C& lo = x[b * B + i];
          C& hi = x[(b | h) * B + i];
          const C s = up ? lo : hi;
          C r;
          r.x = __shfl_xor_sync(0xffffffffu, s.x, h);
          r.y = __shfl_xor_sync(0xffffffffu, s.y, h);
          if (up) lo = r;
          else hi = r;
        }
      }
    }
  }

  // Q2-point DFT over registers p B + i (p = 0..Q2-1) for each i, in place
  template <bool INV> __device__ static __forceinline__ void dft_cols(C (&x)[E]) {
#pragma unroll
    for (int i = 0; i < B; ++i) {
      C t[Q2];
#pragma unroll
      for (int p = 0; p < Q2; ++p) t[p] = x[p * B + i];
      dftE<Q2, INV>(t);
#pragma unroll
      for (int p = 0; p < Q2; ++p) x[p * B + i] = t[p];
    }
  }

  // natural (x[r] = point lane + 32 r) -> a digit-scrambled order, the same
  // for every row and field (E >= Q: x[v B + i] = point k1 + E (q B + i) +
  // E^2 v, with k1 = lane / Q, q = lane % Q)
  // TX: twiddles from the WarpTw tables tx of this M (else powers from the
  // M-point table tw)
  template <bool INV, bool TX = false>
  __device__ static __forceinline__ void nat_to_scr(C (&x)[E], C* sm, const C* __restrict__ tw, int lane,
                                                    const C* __restrict__ tx = nullptr) {
    dftE<E, INV>(x);
    if constexpr (TX) twiddle_first<INV>(x, tx, lane);
    else twiddle_powers<INV>(x, tw, lane);
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) sm[k1 * ROW + lane] = x[k1];
    __syncwarp();
    const int k1 = lane / Q, q = lane % Q;
#pragma unroll
    for (int t = 0; t < E; ++t) x[t] = sm[k1 * ROW + q + Q * t];
    __syncwarp();
    dftE<E, INV>(x);
    if constexpr (TX) twiddle_second<INV>(x, tx, q);
    else twiddle_powers<INV>(x, tw, q * E);
#pragma unroll
    for (int h = Q / 2; h >= HMIN; h >>= 1) {
      const C w = twid(tw, (q & (h - 1)) * (M / (2 * h)), INV);
      const bool up = (q & h) != 0;
#pragma unroll
      for (int u = 0; u < E; ++u) {
        C p;
        p.x = __shfl_xor_sync(0xffffffffu, x[u].x, h);
        p.y = __shfl_xor_sync(0xffffffffu, x[u].y, h);
        x[u] = up ? cmul(csub(p, x[u]), w) : cadd(x[u], p);
      }
    }
    if constexpr (XCH) {
      exchange(x, q);
      dft_cols<INV>(x);
    }
  }

  // scrambled -> natural (the transposed network of nat_to_scr)
  template <bool INV, bool TX = false>
  __device__ static __forceinline__ void scr_to_nat(C (&x)[E], C* sm, const C* __restrict__ tw, int lane,
                                                    const C* __restrict__ tx = nullptr) {
    const int k1 = lane / Q, q = lane % Q;
    if constexpr (XCH) {
      dft_cols<INV>(x);
      exchange(x, q);
    }
#pragma unroll
    for (int h = HMIN; h <= Q / 2; h <<= 1) {
      const C w = twid(tw, (q & (h - 1)) * (M / (2 * h)), INV);
      const bool up = (q & h) != 0;
#pragma unroll
      for (int u = 0; u < E; ++u) {
        C p;
        p.x = __shfl_xor_sync(0xffffffffu, x[u].x, h);
        p.y = __shfl_xor_sync(0xffffffffu, x[u].y, h);
        x[u] = up ? csub(p, cmul(w, x[u])) : cadd(x[u], cmul(w, p));
      }
    }
    if constexpr (TX) twiddle_second<INV>(x, tx, q);
    else twiddle_powers<INV>(x, tw, q * E);
    dftE<E, INV>(x);
#pragma unroll
    for (int t = 0; t < E; ++t) sm[k1 * ROW + q + Q * t] = x[t];
    __syncwarp();
#pragma unroll
    for (int j = 0; j < E; ++j) x[j] = sm[j * ROW + lane];
    __syncwarp();
    if constexpr (TX) twiddle_first<INV>(x, tx, lane);
    else twiddle_powers<INV>(x, tw, lane);
    dftE<E, INV>(x);
  }

  // w[r] = W_N^{lane + 32 r} (N = 2M), r = 0..E-1: one table load times the
  // compile-time roots W_{2E}^r
  __device__ static __forceinline__ void half_twiddles(C (&w)[E], const C* __restrict__ twN, int lane) {
    C cr[E];
    roots::fill<C, 2 * E>(cr, std::make_integer_sequence<int, E>{});
    const C wl = __ldg(&twN[lane]);
    w[0] = wl;
#pragma unroll
    for (int r = 1; r < E; ++r) w[r] = cmul(wl, cr[r]);
  }
};

template <typename T, int LOGM, int MODE = XW_DNS> struct XwCfg {
  // per warp: the transpose buffer + the rows kept in scrambled order (u;
  // XW_SMAG also S_ij)
  static constexpr int KEPT = MODE == XW_SMAG ? 9 : 3;
  // TM: the kept rows in tensor memory instead (FP32; XW_DNS and XW_ADJ at
  // 4 or 8 points per lane, XW_SMAG at 4; SC_XW_NO_TMEM: shared memory):
  // 2 E KEPT columns per warp, two warps per lane quarter, TM_COLS columns
  // per CTA (128, or 256 for the nine XW_SMAG rows)
#ifndef SC_XW_NO_TMEM
  static constexpr bool TM = sizeof(T) == 4 && (MODE != XW_SMAG ? (LOGM == 7 || LOGM == 8) : LOGM == 7);
#else
  static constexpr bool TM = false;
#endif
  static constexpr int TM_COLS = MODE == XW_SMAG ? 256 : 128;
  static constexpr int KEPT_SM = TM ? 0 : KEPT;
  // two staging buffers for the warp's next input rows (points 0 .. M,
  // rounded up to 16 bytes)
  static constexpr int STG = (int)((((WarpFFT<T, LOGM>::M + 1) * sizeof(C2<T>) + 15) / 16 * 16) / sizeof(C2<T>));
#ifdef SC_XW_NO_STAGE
  static constexpr int STAGED = 0;
#else
  static constexpr int STAGED = 2 * STG;
#endif
  static constexpr int PER_WARP = WarpFFT<T, LOGM>::SMEM + KEPT_SM * WarpFFT<T, LOGM>::M + STAGED;
  // the staging buffers are bulk-copy destinations: 16-byte aligned
  static_assert((PER_WARP * sizeof(C2<T>)) % 16 == 0 &&
                    ((WarpFFT<T, LOGM>::SMEM + KEPT_SM * WarpFFT<T, LOGM>::M) * sizeof(C2<T>)) % 16 == 0,
                "x-pass staging buffers must start on 16-byte boundaries");
  // 8 warps per CTA unless that passes 110 KB of shared memory
  static constexpr int WARPS = sizeof(C2<T>) * PER_WARP * 8 <= 110 * 1024 ? 8 : 4;
  static constexpr int NT = 32 * WARPS;
  static_assert(!TM || WARPS == 8 || WARPS == 4, "two lane-quarter blocks of tensor-memory columns at most");
  // CTAs per SM the launch bounds ask for: three (80 registers) where the
  // three rows are in tensor memory and the transforms are 128 points long
  // (no spills), else 16 warps per SM (SC_XW_MINB overrides)
#ifndef SC_XW_MINB
  static constexpr int MINB = (TM && TM_COLS == 128 && LOGM <= 7 && WARPS == 8) ? 3 : 16 / WARPS;
#else
  static constexpr int MINB = SC_XW_MINB;
#endif
  static constexpr size_t SMEM = sizeof(C2<T>) * PER_WARP * WARPS;
  // the launch's shared memory: with 256 tensor-memory columns per CTA, at
  // least 77 KB, so that no more than two CTAs (512 columns) share an SM
  static constexpr size_t SMEM_LAUNCH = (TM && TM_COLS > 128 && SMEM < 77 * 1024) ? 77 * 1024 : SMEM;
};

// One warp's view of one grid row (y, z) at element offset `off` of every
// field.  TM: the a rows in tensor memory.
template <typename T, int LOGM, bool TM = false> struct XwRow {
  using WF = WarpFFT<T, LOGM>;
  using C = C2<T>;
  static constexpr int M = WF::M, E = WF::E;
  static_assert(!TM || (sizeof(T) == 4 && (E == 4 || E == 8)), "tensor-memory rows: FP32, 4 or 8 points per lane");
  C* sm;         // transpose buffer
  C* as;         // three rows a_c at [(c * E + i) * 32 + lane], scrambled order
  uint32_t ta = 0;   // TM: a_c at columns ta + 2 E c .. + 2 E - 1 of the warp's lanes
  const C* twM;
  const C* twN;
  const C* tx = nullptr;   // WarpTw tables of M (used when TX)
#ifndef SC_XW_NO_TX
  static constexpr bool TX = LOGM >= WarpTw::LOGM_MIN && LOGM <= WarpTw::LOGM_MAX;
#else
  static constexpr bool TX = false;
#endif
  long long off;
  int lane;
  // Input rows staged through shared memory: seq lists the fields in the
  // order load_z consumes their rows; while a row is transformed the next
  // one streams into the other buffer (stg == nullptr: load_z reads global
  // memory directly).  Each row arrives by one bulk copy issued by lane 0,
  // completing on the buffer's mbarrier (sbar[0..1]), so the copies take no
  // load/store-unit slots (SC_XW_CPASYNC: 16-byte cp.async by every lane).
  // A wait that gives up records the timeout in *err and the warp waits on
  // nothing after it (its results are then void; the host reports the
  // error).
  C* stg = nullptr;
  int stg_elems = 0;
  const C* const* seq = nullptr;
  int nseq = 0;
  int used = 0;
  uint64_t* sbar = nullptr;
  int* err = nullptr;
  bool ok = true;

  __device__ __forceinline__ void stage_issue(int i) {
    const char* src = reinterpret_cast<const char*>(seq[i] + off);
    char* dst = reinterpret_cast<char*>(stg + (i & 1) * stg_elems);
#ifdef SC_XW_CPASYNC
    const int chunks = stg_elems * (int)sizeof(C) / 16;
    for (int c = lane; c < chunks; c += 32)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                       static_cast<uint32_t>(__cvta_generic_to_shared(dst + 16 * c))),
                   "l"(src + 16 * c)
                   : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
#else
    if (lane == 0) {
      // the buffer's earlier reads (generic proxy) before the copy's writes
      fence_proxy_async();
      const uint32_t bytes = (uint32_t)(stg_elems * sizeof(C));
      mbar_arrive_expect_tx(&sbar[i & 1], bytes);
      bulk_load(dst, src, bytes, &sbar[i & 1]);
    }
#endif
  }
  __device__ __forceinline__ void stage_start() {
#ifndef SC_XW_CPASYNC
    if (lane == 0) {
      mbar_init(&sbar[0], 1);
      mbar_init(&sbar[1], 1);
      fence_mbar_init();
    }
    __syncwarp();
#endif
    stage_issue(0);
    if (nseq > 1) stage_issue(1);
  }
  // the row of seq[used], staged and visible to the whole warp
  __device__ __forceinline__ const C* stage_acquire() {
#ifdef SC_XW_CPASYNC
    if (used + 1 < nseq) asm volatile("cp.async.wait_group 1;" ::: "memory");
    else asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncwarp();
#else
    // buffer b's k-th fill (row index i = 2k + b) completes phase k
    if (ok) ok = mbar_wait_bounded(&sbar[used & 1], (uint32_t)(used >> 1) & 1u, err);
#endif
    return stg + (used & 1) * stg_elems;
  }
  // every lane is done with that row: its buffer takes the row after next
  __device__ __forceinline__ void stage_release() {
    __syncwarp();
    if (used + 2 < nseq && ok) stage_issue(used + 2);
    ++used;
  }

  // wn[r] = W_N^{lane + 32 r}, N = 2M: one table load times compile-time
  // roots (SC_XW_HALFLOAD: one table load each)
  __device__ __forceinline__ void half_twiddles(C (&wn)[E]) const {
#ifdef SC_XW_HALFLOAD
#pragma unroll
    for (int r = 0; r < E; ++r) wn[r] = __ldg(&twN[lane + 32 * r]);
#else
    WF::half_twiddles(wn, twN, lane);
#endif
  }

  // half-length c2r pre-processing of a row into natural-order Z
  __device__ __forceinline__ void load_z(const C* __restrict__ fp, C (&x)[E]) {
    const C* __restrict__ rp = stg ? stage_acquire() : fp + off;
    C wn[E];
    half_twiddles(wn);
#pragma unroll
    for (int r = 0; r < E; ++r) {
      const int k = lane + 32 * r;
      C xk = rp[k], xm = rp[M - k];
      if (k == 0) { xk.y = 0; xm.y = 0; }   // DC and Nyquist are real
      const C e = cadd(xk, cconj(xm));
      const C o = cmulc(csub(xk, cconj(xm)), wn[r]);
      x[r] = cadd(e, cmuli(o));
    }
    if (stg) stage_release();
  }

  // a_c = c2r of rows f[0..2], kept in shared memory
  __device__ __forceinline__ void load_a(const C* const f[3]) {
#pragma unroll 1
    for (int c = 0; c < 3; ++c) {
      C x[E];
      load_z(f[c], x);
      WF::template nat_to_scr<true, TX>(x, sm, twM, lane, tx);
      if constexpr (TM) {
        uint32_t w[2 * E];
#pragma unroll
        for (int i = 0; i < E; ++i) {
          w[2 * i] = __float_as_uint(x[i].x);
          w[2 * i + 1] = __float_as_uint(x[i].y);
        }
        if constexpr (E == 8) tmem_store16(ta + 16u * c, w);
        else tmem_store8(ta + 8u * c, w);
      } else {
#pragma unroll
        for (int i = 0; i < E; ++i) as[(c * E + i) * 32 + lane] = x[i];
      }
    }
    if constexpr (TM) tmem_wait_store();
  }

  // a_c at points i0 .. i0+3
  __device__ __forceinline__ void a4(int c, int i0, C (&a)[4]) const {
    if constexpr (TM) {
      uint32_t w[8];
      tmem_load8(ta + (uint32_t)(2 * E * c + 2 * i0), w);
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = mk<C>(__uint_as_float(w[2 * i]), __uint_as_float(w[2 * i + 1]));
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = as[(c * E + i0 + i) * 32 + lane];
    }
  }

  // r2c post-processing of natural-order Z into the half-complex row at op:
  // needs Z_{M-k}; k = lane + 32 r pairs with lane (32 - lane) % 32,
  // register E-1-r (lane 0: its own register (E - r) % E)
  __device__ __forceinline__ void r2c_store(C (&x)[E], C* __restrict__ op) const {
    const int src = (32 - lane) & 31;
    C wn[E];
    half_twiddles(wn);
#pragma unroll
    for (int r = 0; r < E; ++r) {
      C zm;
      zm.x = __shfl_sync(0xffffffffu, x[E - 1 - r].x, src);
      zm.y = __shfl_sync(0xffffffffu, x[E - 1 - r].y, src);
      if (lane == 0) zm = x[(E - r) % E];
      const int k = lane + 32 * r;
      const C zk = x[r];
      const C zmc = cconj(zm);
      const C e = cadd(zk, zmc);
      const C d = cmul(csub(zk, zmc), wn[r]);
      op[k] = cscale(csub(e, cmuli(d)), T(0.5));
      if (k == 0) {   // X_M from Z_0
        const C d0 = cmul(csub(zk, zmc), __ldg(&twN[M]));
        op[M] = cscale(csub(e, cmuli(d0)), T(0.5));
      }
    }
  }

  // out = r2c(sc * (a x b)), b = c2r of rows bf[0..2]; the cross product is
  // accumulated as the b components arrive (convec_dns.f90:30-38: even
  // points in .x, odd points in .y)
  __device__ __forceinline__ void cross_store(const C* const bf[3], C* const of[3], T sc) {
    static_assert(E % 4 == 0 || !TM, "a rows are read four points at a time");
    constexpr int G = E < 4 ? E : 4;   // points per group of a reads
    auto A = [&](int c, int i0, C (&a)[4]) {
      if constexpr (TM) a4(c, i0, a);
      else {
#pragma unroll
        for (int i = 0; i < G; ++i) a[i] = as[(c * E + i0 + i) * 32 + lane];
      }
    };
    // L_z is complete after b_y and leaves before b_z is transformed, so
    // only L_x and L_y stay in registers through the last transform
    auto out = [&](C (&l)[E], int c) {
      C x[E];
#pragma unroll
      for (int i = 0; i < E; ++i) x[i] = cscale(l[i], sc);
      WF::template scr_to_nat<false, TX>(x, sm, twM, lane, tx);
      r2c_store(x, of[c] + off);
    };
    C l0[E], l1[E];
    C b[E];
    {
      C l2[E];
      load_z(bf[0], b);   // b_x: L_y = a_z b_x - ..., L_z = ... - a_y b_x
      WF::template nat_to_scr<true, TX>(b, sm, twM, lane, tx);
#pragma unroll
      for (int i0 = 0; i0 < E; i0 += G) {
        C a1[4], a2[4];
        A(1, i0, a1);
        A(2, i0, a2);
#pragma unroll
        for (int ii = 0; ii < G; ++ii) {
          const int i = i0 + ii;
          l1[i] = mk<C>(a2[ii].x * b[i].x, a2[ii].y * b[i].y);
          l2[i] = mk<C>(-(a1[ii].x * b[i].x), -(a1[ii].y * b[i].y));
        }
      }
      load_z(bf[1], b);   // b_y: L_x = ... - a_z b_y, L_z = a_x b_y - a_y b_x
      WF::template nat_to_scr<true, TX>(b, sm, twM, lane, tx);
#pragma unroll
      for (int i0 = 0; i0 < E; i0 += G) {
        C a0[4], a2[4];
        A(0, i0, a0);
        A(2, i0, a2);
#pragma unroll
        for (int ii = 0; ii < G; ++ii) {
          const int i = i0 + ii;
          l0[i] = mk<C>(-(a2[ii].x * b[i].x), -(a2[ii].y * b[i].y));
          l2[i] = mk<C>(a0[ii].x * b[i].x + l2[i].x, a0[ii].y * b[i].y + l2[i].y);
        }
      }
      out(l2, 2);
    }
    load_z(bf[2], b);   // b_z: L_x = a_y b_z - a_z b_y, L_y = a_z b_x - a_x b_z
    WF::template nat_to_scr<true, TX>(b, sm, twM, lane, tx);
#pragma unroll
    for (int i0 = 0; i0 < E; i0 += G) {
      C a0[4], a1[4];
      A(0, i0, a0);
      A(1, i0, a1);
#pragma unroll
      for (int ii = 0; ii < G; ++ii) {
        const int i = i0 + ii;
        l0[i] = mk<C>(a1[ii].x * b[i].x + l0[i].x, a1[ii].y * b[i].y + l0[i].y);
        l1[i] = mk<C>(l1[i].x - a0[ii].x * b[i].x, l1[i].y - a0[ii].y * b[i].y);
      }
    }
    out(l0, 0);
    out(l1, 1);
  }

  // S_ij rows sf[0..5] (order 11 12 13 22 23 33) -> c2r, kept in shared
  // memory after the three a rows
  __device__ __forceinline__ void load_s(const C* const sf[6]) {
#pragma unroll 1
    for (int q = 0; q < 6; ++q) {
      C x[E];
      load_z(sf[q], x);
      WF::template nat_to_scr<true, TX>(x, sm, twM, lane, tx);
#pragma unroll
      if constexpr (TM) {
        uint32_t w[2 * E];
#pragma unroll
        for (int i = 0; i < E; ++i) {
          w[2 * i] = __float_as_uint(x[i].x);
          w[2 * i + 1] = __float_as_uint(x[i].y);
        }
        if constexpr (E == 4) tmem_store8(ta + 8u * (3 + q), w);
      } else {
#pragma unroll
        for (int i = 0; i < E; ++i) as[((3 + q) * E + i) * 32 + lane] = x[i];
      }
    }
    if constexpr (TM) tmem_wait_store();
  }

  // tau_ij = tcoef |S| S_ij on every real point (smag.f90:41-64: even points
  // in .x, odd in .y), |S| = sqrt(2 (S11^2 + S22^2 + S33^2 + 2 (S12^2 + S13^2
  // + S23^2))); r2c into of[0..5]
  __device__ __forceinline__ void tau_store(C* const of[6], T tcoef) const {
    if constexpr (TM) {
      // rows from tensor memory one at a time: the diagonal and off-diagonal
      // sums in the order of the shared-memory form below
      static_assert(E == 4, "tensor-memory S rows: 4 points per lane");
      T dx[E], dy[E], ox[E], oy[E], ar[E], ai[E];
      C r[4];
      auto acc = [&](int q, T (&sx)[E], T (&sy)[E], bool first) {
        a4(3 + q, 0, r);
#pragma unroll
        for (int i = 0; i < E; ++i) {
          sx[i] = first ? r[i].x * r[i].x : sx[i] + r[i].x * r[i].x;
          sy[i] = first ? r[i].y * r[i].y : sy[i] + r[i].y * r[i].y;
        }
      };
      acc(0, dx, dy, true);    // S11
      acc(3, dx, dy, false);   // S22
      acc(5, dx, dy, false);   // S33
      acc(1, ox, oy, true);    // S12
      acc(2, ox, oy, false);   // S13
      acc(4, ox, oy, false);   // S23
#pragma unroll
      for (int i = 0; i < E; ++i) {
        ar[i] = tcoef * sqrt(T(2) * (dx[i] + T(2) * ox[i]));
        ai[i] = tcoef * sqrt(T(2) * (dy[i] + T(2) * oy[i]));
      }
#pragma unroll 1
      for (int q = 0; q < 6; ++q) {
        a4(3 + q, 0, r);
        C x[E];
#pragma unroll
        for (int i = 0; i < E; ++i) x[i] = mk<C>(ar[i] * r[i].x, ai[i] * r[i].y);
        WF::template scr_to_nat<false, TX>(x, sm, twM, lane, tx);
        r2c_store(x, of[q] + off);
      }
      return;
    }
    auto S = [&](int q, int i) { return as[((3 + q) * E + i) * 32 + lane]; };
    T ar[E], ai[E];
#pragma unroll
    for (int i = 0; i < E; ++i) {
      const C s11 = S(0, i), s12 = S(1, i), s13 = S(2, i), s22 = S(3, i), s23 = S(4, i), s33 = S(5, i);
      ar[i] = tcoef * sqrt(T(2) * (s11.x * s11.x + s22.x * s22.x + s33.x * s33.x +
                                   T(2) * (s12.x * s12.x + s13.x * s13.x + s23.x * s23.x)));
      ai[i] = tcoef * sqrt(T(2) * (s11.y * s11.y + s22.y * s22.y + s33.y * s33.y +
                                   T(2) * (s12.y * s12.y + s13.y * s13.y + s23.y * s23.y)));
    }
#pragma unroll 1
    for (int q = 0; q < 6; ++q) {
      C x[E];
#pragma unroll
      for (int i = 0; i < E; ++i) {
        const C s = S(q, i);
        x[i] = mk<C>(ar[i] * s.x, ai[i] * s.y);
      }
      WF::template scr_to_nat<false, TX>(x, sm, twM, lane, tx);
      r2c_store(x, of[q] + off);
    }
  }
};

// XW_DNS: fin = (u, w) -> fout[0..2] = r2c(u x w / N^3), in place allowed.
// XW_SMAG: fin = (u, w, S_ij) -> fout[0..2] = r2c(u x w / N^3) and
//   fout[3..8] = r2c(tau_ij), tau_ij = -2 c1 D^2 |S| S_ij / N^3 (smag.f90:41-64),
//   in place allowed: u and S are staged and w is read before any output.
// XW_ADJ: fin = (u, w, phi) -> adjoint of the Lamb product (no scale):
//   w x phi = -(phi x w) into fout[0..2], then phi x u into fout[3..5];
//   fout must not alias u (read by the second product) -- the host passes
//   the w and phi slots.
template <typename T, int LOGM, int MODE>
__global__ void __launch_bounds__(XwCfg<T, LOGM, MODE>::NT, XwCfg<T, LOGM, MODE>::MINB)
xpass_warp_kernel(FieldList<T> fin, FieldList<T> fout, Geom g, const C2<T>* __restrict__ twM,
                  const C2<T>* __restrict__ twN, XArgs<T> xa) {
  using C = C2<T>;
  using Cfg = XwCfg<T, LOGM, MODE>;
  using Row = XwRow<T, LOGM, Cfg::TM>;
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ __align__(8) uint64_t sbar[2 * Cfg::WARPS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long long row = (long long)blockIdx.x * Cfg::WARPS + warp;
  // TM: the CTA's TM_COLS columns, warp w at lanes 32 (w % 4), columns
  // TM_COLS / 2 * (w / 4)
  __shared__ uint32_t s_tmem;
  if constexpr (Cfg::TM) {
    if (warp == 0) tmem_alloc(&s_tmem, Cfg::TM_COLS);
    tmem_fence_before_sync();
    __syncthreads();
    tmem_fence_after_sync();
  } else {
    if (row >= xa.rows) return;
  }
  if (row < xa.rows) {
    Row R;
    R.sm = reinterpret_cast<C*>(smraw) + warp * Cfg::PER_WARP;
    R.as = R.sm + WarpFFT<T, LOGM>::SMEM;
    if constexpr (Cfg::TM)
      R.ta = s_tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(Cfg::TM_COLS / 2) * (uint32_t)(warp >> 2);
    R.twM = twM;
    R.twN = twN;
    if constexpr (Row::TX) R.tx = xa.twx + WarpTw::offset(LOGM);
    R.off = row * g.nxp;
    R.lane = lane;
    // the input fields in the order their rows are consumed
    const C* seq[Cfg::KEPT == 9 ? 12 : (MODE == XW_ADJ ? 9 : 6)];
    if constexpr (MODE == XW_DNS) {
      for (int f = 0; f < 6; ++f) seq[f] = fin.f[f];
    } else if constexpr (MODE == XW_SMAG) {
      for (int f = 0; f < 3; ++f) seq[f] = fin.f[f];          // u (load_a)
      for (int f = 0; f < 6; ++f) seq[3 + f] = fin.f[6 + f];  // S_ij (load_s)
      for (int f = 0; f < 3; ++f) seq[9 + f] = fin.f[3 + f];  // w (cross_store)
    } else {
      for (int f = 0; f < 3; ++f) seq[f] = fin.f[6 + f];      // phi (load_a)
      for (int f = 0; f < 3; ++f) seq[3 + f] = fin.f[3 + f];  // w
      for (int f = 0; f < 3; ++f) seq[6 + f] = fin.f[f];      // u
    }
    if constexpr (Cfg::STAGED > 0) {
      R.stg = R.sm + WarpFFT<T, LOGM>::SMEM + Cfg::KEPT_SM * WarpFFT<T, LOGM>::M;
      R.stg_elems = Cfg::STG;
      R.seq = seq;
      R.nseq = (int)(sizeof(seq) / sizeof(seq[0]));
      R.sbar = sbar + 2 * warp;
      R.err = xa.err;
      R.stage_start();
    }
    if constexpr (MODE == XW_DNS) {
      const C* a[3] = {fin.f[0], fin.f[1], fin.f[2]};
      const C* b[3] = {fin.f[3], fin.f[4], fin.f[5]};
      C* o[3] = {fout.f[0], fout.f[1], fout.f[2]};
      R.load_a(a);
      R.cross_store(b, o, xa.scale);
    } else if constexpr (MODE == XW_SMAG) {
      const C* a[3] = {fin.f[0], fin.f[1], fin.f[2]};
      const C* b[3] = {fin.f[3], fin.f[4], fin.f[5]};
      const C* s[6] = {fin.f[6], fin.f[7], fin.f[8], fin.f[9], fin.f[10], fin.f[11]};
      C* o[3] = {fout.f[0], fout.f[1], fout.f[2]};
      C* ot[6] = {fout.f[3], fout.f[4], fout.f[5], fout.f[6], fout.f[7], fout.f[8]};
      const T tcoef = (T)(-2.0 * (*xa.c1) * xa.delta2) * xa.scale;
      R.load_a(a);
      R.load_s(s);
      R.cross_store(b, o, xa.scale);
      R.tau_store(ot, tcoef);
    } else {
      const C* phi[3] = {fin.f[6], fin.f[7], fin.f[8]};
      const C* w[3] = {fin.f[3], fin.f[4], fin.f[5]};
      const C* u[3] = {fin.f[0], fin.f[1], fin.f[2]};
      C* o1[3] = {fout.f[0], fout.f[1], fout.f[2]};
      C* o2[3] = {fout.f[3], fout.f[4], fout.f[5]};
      R.load_a(phi);
      R.cross_store(w, o1, T(-1));
      R.cross_store(u, o2, T(1));
    }
  }
  if constexpr (Cfg::TM) {
    // every warp's tensor-memory reads are complete before the release
    tmem_fence_before_sync();
    __syncthreads();
    if (warp == 0) {
      tmem_fence_after_sync();
      tmem_dealloc(s_tmem, Cfg::TM_COLS);
    }
  }
}

}  // namespace sc
