// Block-level batched FFT engine for sm_103a.
//
// A thread block transforms P independent pencils of length N = 2^LOGN held
// in shared memory as sm[n*PS + p] (pencil p, point n).  The transform is a
// Stockham autosort FFT (radix-8 stages, then radix-4/2 to finish), so the
// output comes out in natural order without a bit-reversal pass.
//
// The first stage takes its inputs straight from registers and the last stage
// leaves its outputs in registers, so a pass that loads from HBM, transforms
// and stores back touches shared memory only for the exchanges between
// stages.  Input element (p, n) for register slot in[a][r] is
//     job = threadIdx.x + a*NT, (p, j) = decode(job), n = j + r*(N/R1)
// and output slot out[a][r] holds element n = j + r*(N/RL) of pencil p, with
// decode giving p fastest (PFAST: consecutive threads walk consecutive
// pencils, the layout of strided-axis passes whose pencils are contiguous in
// HBM) or j fastest (consecutive threads walk one pencil, the layout of the
// x-axis pass whose pencils are HBM rows).
//
// Twiddles W_N^m = exp(-2 pi i m/N) come from a table computed in double on
// the host and rounded once to T.  Forward = exp(-i..), inverse = exp(+i..),
// both unnormalised (FFTW's convention).
#pragma once
#include "sc_common.cuh"

namespace sc {

// Radix plan.  rmax = 8: as many radix-8 stages as possible, finished by one
// radix-4 (LOGN % 3 == 2), two radix-4 (LOGN % 3 == 1) or a lone radix-2
// (N = 2).  rmax = 4: radix-4 stages, the last one radix-2 for odd LOGN
// (half the registers per butterfly job, one more pass over shared memory).
__host__ __device__ constexpr int fft_nstages(int logn, int rmax = 8) {
  return rmax == 4 ? (logn + 1) / 2 : (logn <= 3 ? 1 : (logn % 3 == 0 ? logn / 3 : logn / 3 + 1));
}
__host__ __device__ constexpr int fft_radix(int logn, int s, int rmax = 8) {
  return rmax == 4 ? ((logn & 1) && s == fft_nstages(logn, 4) - 1 ? 2 : 4)
       : logn == 1 ? 2
       : logn == 2 ? 4
       : logn % 3 == 0 ? 8
       : logn % 3 == 2 ? (s < logn / 3 ? 8 : 4)
       : (s < logn / 3 - 1 ? 8 : 4);
}
__host__ __device__ constexpr int fft_ns(int logn, int s, int rmax = 8) {
  return s == 0 ? 1 : fft_ns(logn, s - 1, rmax) * fft_radix(logn, s - 1, rmax);
}

template <typename T> struct Consts;
template <> struct Consts<float> { static constexpr float rsqrt2 = 0.70710678118654752440f; };
template <> struct Consts<double> { static constexpr double rsqrt2 = 0.70710678118654752440; };

template <bool INV, typename C> __device__ __forceinline__ void dft2(C* v) {
  C t = v[0];
  v[0] = cadd(t, v[1]);
  v[1] = csub(t, v[1]);
}

template <bool INV, typename C> __device__ __forceinline__ void dft4(C* v) {
  C t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
  C t2 = cadd(v[1], v[3]), t3 = csub(v[1], v[3]);
  t3 = INV ? cmuli(t3) : cmulmi(t3);
  v[0] = cadd(t0, t2);
  v[2] = csub(t0, t2);
  v[1] = cadd(t1, t3);
  v[3] = csub(t1, t3);
}

template <bool INV, typename C> __device__ __forceinline__ void dft8(C* v) {
  using R = decltype(C::x);
  const R h = Consts<R>::rsqrt2;
  C e[4] = {v[0], v[2], v[4], v[6]};
  C o[4] = {v[1], v[3], v[5], v[7]};
  dft4<INV>(e);
  dft4<INV>(o);
  // o[k] *= W_8^{+-k}
  if (INV) {
    o[1] = mk<C>((o[1].x - o[1].y) * h, (o[1].x + o[1].y) * h);
    o[2] = cmuli(o[2]);
    o[3] = mk<C>((-o[3].x - o[3].y) * h, (o[3].x - o[3].y) * h);
  } else {
    o[1] = mk<C>((o[1].x + o[1].y) * h, (o[1].y - o[1].x) * h);
    o[2] = cmulmi(o[2]);
    o[3] = mk<C>((o[3].y - o[3].x) * h, (-o[3].x - o[3].y) * h);
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd(e[k], o[k]);
    v[k + 4] = csub(e[k], o[k]);
  }
}

template <typename R> struct W16;
template <> struct W16<float> {
  static constexpr float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;
  static constexpr float h = 0.70710678118654752440f;
};
template <> struct W16<double> {
  static constexpr double c1 = 0.92387953251128675613, s1 = 0.38268343236508977173;
  static constexpr double h = 0.70710678118654752440;
};

// 16-point DFT in registers as 4 x 4 (n = n1 + 4 n2, k = k2 + 4 k1), in
// place: radix-4 over n2 for each n1, twiddles W16^{n1 k2}, radix-4 over n1
// for each k2, then a 4 x 4 register transpose into natural order.
template <bool INV, typename C> __device__ __forceinline__ void dft16(C* v) {
  using R = decltype(C::x);
#pragma unroll
  for (int n1 = 0; n1 < 4; ++n1) {
    C t[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
    dft4<INV>(t);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) v[n1 + 4 * k2] = t[k2];
  }
#pragma unroll
  for (int n1 = 1; n1 < 4; ++n1)
#pragma unroll
    for (int k2 = 1; k2 < 4; ++k2) {
      const int e = n1 * k2;
      R c, sn;   // W16^e = cos(2 pi e/16) - i sin(2 pi e/16) (forward)
      switch (e) {
        case 1: c = W16<R>::c1; sn = W16<R>::s1; break;
        case 2: c = W16<R>::h; sn = W16<R>::h; break;
        case 3: c = W16<R>::s1; sn = W16<R>::c1; break;
        case 4: c = 0; sn = 1; break;
        case 6: c = -W16<R>::h; sn = W16<R>::h; break;
        default: c = -W16<R>::c1; sn = -W16<R>::s1; break;   // e = 9
      }
      v[n1 + 4 * k2] = cmul(v[n1 + 4 * k2], mk<C>(c, INV ? sn : -sn));
    }
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) dft4<INV>(v + 4 * k2);   // X[k2 + 4 k1] now at v[k1 + 4 k2]
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = i + 1; j < 4; ++j) {
      const C t = v[j + 4 * i];
      v[j + 4 * i] = v[i + 4 * j];
      v[i + 4 * j] = t;
    }
}

template <int R, bool INV, typename C> __device__ __forceinline__ void dft(C* v) {
  if constexpr (R == 2) dft2<INV>(v);
  else if constexpr (R == 4) dft4<INV>(v);
  else dft8<INV>(v);
}

template <typename T, int LOGN, int P, int PS, int NT, bool PFAST, int PADSHIFT = 0, bool ROTATE = false,
          int RMAX = 8>
struct FFTEngine {
  using C = C2<T>;
  static constexpr int N = 1 << LOGN;
  static constexpr int NS = fft_nstages(LOGN, RMAX);
  static constexpr int R1 = fft_radix(LOGN, 0, RMAX);
  static constexpr int RL = fft_radix(LOGN, NS - 1, RMAX);
  static constexpr int TOT1 = P * (N / R1);
  static constexpr int TOTL = P * (N / RL);
  static constexpr int J1 = (TOT1 + NT - 1) / NT;
  static constexpr int JL = (TOTL + NT - 1) / NT;
  // Shared-memory slot of point n.  With PADSHIFT = s one slot is skipped
  // every 2^s points, which spreads the stride-R scatter of the first stage
  // over all banks: s = 4 keeps both that scatter and 16-wide contiguous
  // runs conflict-free for pencil-per-warp (j-fastest) layouts with odd PS;
  // s = 3 does it for 8-wide p-fastest tiles (64-byte rows).
  static constexpr int NPAD = PADSHIFT ? N + (N >> PADSHIFT) : N;
  static constexpr int SMEM_ELEMS = NPAD * PS;
  __device__ static __forceinline__ int sidx(int n) { return PADSHIFT ? n + (n >> PADSHIFT) : n; }

  template <int R>
  __device__ static __forceinline__ void decode(int job, int& p, int& j) {
    constexpr int NR = N / R;
    if constexpr (PFAST) {
      p = job % P;
      j = job / P;
    } else {
      j = job % NR;
      p = job / NR;
    }
  }
  // Position of in[a][r]; returns false for padding jobs.
  __device__ static __forceinline__ bool in_pos(int a, int r, int& p, int& n) {
    int job = threadIdx.x + a * NT, j;
    decode<R1>(job, p, j);
    n = j + r * (N / R1);
    return (TOT1 % NT == 0) || job < TOT1;
  }
  // Position of out[a][r]; returns false for padding jobs.
  __device__ static __forceinline__ bool out_pos(int a, int r, int& p, int& n) {
    int job = threadIdx.x + a * NT, j;
    decode<RL>(job, p, j);
    n = j + r * (N / RL);
    return (TOTL % NT == 0) || job < TOTL;
  }

  // Stage-0 writes go to rows j*R + r.  With p fastest, the 32/P jobs of a
  // warp write rows R apart; for rows narrower than the 128-byte bank window
  // and r the same across the warp they all fall in one part of the window
  // (a 4-way conflict for 64-byte rows).  Each job therefore writes its rows
  // in the order r ^ m, m = j mod (rows per window), which spreads the warp
  // over the whole window; the values are permuted in registers to match.
  // Opt-in (ROTATE): the selects cost registers and issue slots, which the
  // 64-register pencil passes cannot spare.
  static constexpr int ROWB = PS * (int)sizeof(C);
  static constexpr int WIN = (ROTATE && PFAST && PADSHIFT == 0 && ROWB < 128 && 32 % P == 0) ? 128 / ROWB : 1;
  template <int R>
  __device__ static __forceinline__ void store_stage0(C (&v)[R], C* sm, int j, int p) {
    constexpr int W = WIN < R ? WIN : R;
    if constexpr (W > 1) {
      const int m = j & (W - 1);
#pragma unroll
      for (int b = 1; b < W; b <<= 1) {
        const bool sw = (m & b) != 0;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (!(r & b)) {
            const C lo = v[r], hi = v[r | b];
            v[r] = sw ? hi : lo;
            v[r | b] = sw ? lo : hi;
          }
      }
#pragma unroll
      for (int r = 0; r < R; ++r) sm[sidx(j * R + (r ^ m)) * PS + p] = v[r];
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) sm[sidx(j * R + r) * PS + p] = v[r];
    }
  }

  template <int R, int NSV, bool INV>
  __device__ static __forceinline__ void twiddle(C* v, int k, const C* __restrict__ tw) {
    if constexpr (NSV > 1) {
      constexpr int STRIDE = N / (NSV * R);
#pragma unroll
      for (int r = 1; r < R; ++r) {
        C w = __ldg(&tw[k * r * STRIDE]);
        v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
      }
    }
  }

  // The same in two steps: the table loads are issued with the stage's
  // shared-memory reads, before its barrier, so their latency overlaps the
  // barrier wait (SC_TW_LATE: loads after the barrier, as `twiddle`).
#ifdef SC_TW_LATE
  static constexpr bool TW_EARLY = false;
#else
  static constexpr bool TW_EARLY = true;
#endif
  template <int R, int NSV>
  __device__ static __forceinline__ void twiddle_load(C* w, int k, const C* __restrict__ tw) {
    if constexpr (NSV > 1) {
      constexpr int STRIDE = N / (NSV * R);
#pragma unroll
      for (int r = 1; r < R; ++r) w[r] = __ldg(&tw[k * r * STRIDE]);
    }
  }
  template <int R, int NSV, bool INV>
  __device__ static __forceinline__ void twiddle_apply(C* v, const C* w) {
    if constexpr (NSV > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = INV ? cmulc(v[r], w[r]) : cmul(v[r], w[r]);
    }
  }

  // Stage S (0 < S < NS-1): shared -> shared.
  template <int S, bool INV>
  __device__ static __forceinline__ void mid_stage(C* sm, const C* __restrict__ tw) {
    constexpr int R = fft_radix(LOGN, S, RMAX);
    constexpr int NR = N / R;
    constexpr int NSV = fft_ns(LOGN, S, RMAX);
    constexpr int TOT = P * NR;
    constexpr int J = (TOT + NT - 1) / NT;
    C v[J][R], w[TW_EARLY && NSV > 1 ? J : 1][R];
#pragma unroll
    for (int a = 0; a < J; ++a) {
      int job = threadIdx.x + a * NT, p, j;
      decode<R>(job, p, j);
      if ((TOT % NT == 0) || job < TOT) {
#pragma unroll
        for (int r = 0; r < R; ++r) v[a][r] = sm[sidx(j + r * NR) * PS + p];
        if constexpr (TW_EARLY && NSV > 1) twiddle_load<R, NSV>(w[a], j % NSV, tw);
      }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < J; ++a) {
      int job = threadIdx.x + a * NT, p, j;
      decode<R>(job, p, j);
      if ((TOT % NT == 0) || job < TOT) {
        const int k = j % NSV;
        if constexpr (TW_EARLY && NSV > 1) twiddle_apply<R, NSV, INV>(v[a], w[a]);
        else twiddle<R, NSV, INV>(v[a], k, tw);
        dft<R, INV>(v[a]);
        if constexpr (S == 0) {
          store_stage0<R>(v[a], sm, j, p);
        } else {
          const int d = (j / NSV) * NSV * R + k;
#pragma unroll
          for (int r = 0; r < R; ++r) sm[sidx(d + r * NSV) * PS + p] = v[a][r];
        }
      }
    }
    __syncthreads();
  }

  template <int S, bool INV>
  __device__ static __forceinline__ void mid_stages(C* sm, const C* __restrict__ tw) {
    if constexpr (S < NS - 1) {
      mid_stage<S, INV>(sm, tw);
      mid_stages<S + 1, INV>(sm, tw);
    }
  }

  template <int S, bool INV>
  __device__ static __forceinline__ void all_stages(C* sm, const C* __restrict__ tw) {
    if constexpr (S < NS) {
      mid_stage<S, INV>(sm, tw);
      all_stages<S + 1, INV>(sm, tw);
    }
  }

  // Last stage: shared -> registers (last-stage layout).
  template <bool INV>
  __device__ static __forceinline__ void last_stage(C (&out)[JL][RL], C* sm, const C* __restrict__ tw) {
    constexpr int NR = N / RL;
    constexpr int NSV = fft_ns(LOGN, NS - 1, RMAX);
    static_assert(NSV == NR, "last stage spans the pencil");
    C w[TW_EARLY && NSV > 1 ? JL : 1][RL];
#pragma unroll
    for (int a = 0; a < JL; ++a) {
      int job = threadIdx.x + a * NT, p, j;
      decode<RL>(job, p, j);
      if ((TOTL % NT == 0) || job < TOTL) {
#pragma unroll
        for (int r = 0; r < RL; ++r) out[a][r] = sm[sidx(j + r * NR) * PS + p];
        if constexpr (TW_EARLY && NSV > 1) twiddle_load<RL, NSV>(w[a], j, tw);
      }
    }
    __syncthreads();
#pragma unroll
    for (int a = 0; a < JL; ++a) {
      int job = threadIdx.x + a * NT, p, j;
      decode<RL>(job, p, j);
      if ((TOTL % NT == 0) || job < TOTL) {
        if constexpr (TW_EARLY && NSV > 1) twiddle_apply<RL, NSV, INV>(out[a], w[a]);
        else twiddle<RL, NSV, INV>(out[a], j, tw);
        dft<RL, INV>(out[a]);
      }
    }
  }

  // Input already in shared memory (natural order), output in registers.
  // Ends with a barrier.
  template <bool INV>
  __device__ static void run_smem(C (&out)[JL][RL], C* sm, const C* __restrict__ tw) {
    mid_stages<0, INV>(sm, tw);
    last_stage<INV>(out, sm, tw);
  }

  // N = 512 with 32 threads per pencil (NT = 32 P, 16 points each): two
  // passes, 512 = 16 x 32, instead of three radix-8 stages.  Thread (p, j),
  // p = t % P, j = t / P:
  //  1. a 16-point DFT over x[j + 32 m] (m = 0..15) and the twiddles
  //     W512^(j k1): Y[k1][j];
  //  2. Y[k1][j] to row k1 * 32 + (j ^ (k1 & 1)) (the exchange);
  //  3. thread (p, j) with k1 = (j & 1) | (j / 4) * 2, e = (j / 2) & 1
  //     takes the 16 points Y[k1][2 m + e]: a 16-point DFT gives A_e[k'],
  //     and X[k1 + 16 k2] = A_0[k'] +- W32^k' A_1[k'] (k2 = k' or k' + 16)
  //     is finished across the lane pair (lane ^ 2P), each lane keeping
  //     eight k'.
  // The pairing and the row swizzle put the two 64-byte rows that each
  // half-warp (8-byte elements) or quarter-warp (16-byte elements) touches in
  // opposite halves of the banks, so every phase is free of bank conflicts;
  // the transform takes three barriers instead of six.
  static constexpr bool TWO_PASS = PFAST && PS == P && PADSHIFT == 0 && RMAX == 8 &&
                                   ((LOGN == 9 && NT == 32 * P && P <= 8 && 32 % P == 0) ||
                                    (LOGN == 8 && NT == 16 * P && (32 % P == 0 || P % 32 == 0)));
  // N = 256 takes the same two passes as 16 x 16: step 1 as for 512 (points
  // j + 16 m), the exchange at row k1 * 16 + j, and thread (p, k1) finishes
  // the 16-point DFT over j alone (no lane pairs); rows of 8 or 16 elements
  // are whole 128-byte lines, so every access is conflict-free.
  static constexpr int S1 = N / 16;   // stride of the step-1 points
  // Step 1 on values in registers: v[m] = x[j + S1 m] of this thread's
  // pencil p and column j on entry, Y[k1][j] = W_N^(j k1) DFT16(v)[k1] on
  // return (the names say 512; N = 256 uses them too).
  template <bool INV>
  __device__ static __forceinline__ void phase1_512(C (&v)[16], const C* __restrict__ tw) {
    const int j = threadIdx.x / P;
    dft16<INV>(v);
#pragma unroll
    for (int k1 = 1; k1 < 16; ++k1) {
      const C w = __ldg(&tw[j * k1]);
      v[k1] = INV ? cmulc(v[k1], w) : cmul(v[k1], w);
    }
  }

  // Steps 2 and 3 from the step-1 values in registers, through the tile sm
  // (whose previous contents every thread must be done with), leaving the
  // transform in sm in natural order.  Ends with a barrier.
  template <bool INV>
  __device__ static __forceinline__ void finish_512(C (&v)[16], C* sm, const C* __restrict__ tw) {
    const int t = threadIdx.x;
    const int p = t % P, j = t / P;
    if constexpr (LOGN == 8) {
#pragma unroll
      for (int k1 = 0; k1 < 16; ++k1) sm[(k1 * 16 + j) * PS + p] = v[k1];
      __syncthreads();
      // thread (p, k1 = j): the 16-point DFT over the exchange row's j
#pragma unroll
      for (int m = 0; m < 16; ++m) v[m] = sm[(j * 16 + m) * PS + p];
      dft16<INV>(v);
      __syncthreads();
#pragma unroll
      for (int k2 = 0; k2 < 16; ++k2) sm[(j + 16 * k2) * PS + p] = v[k2];
      __syncthreads();
      return;
    }
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) sm[(k1 * 32 + (j ^ (k1 & 1))) * PS + p] = v[k1];
    __syncthreads();
    const int k1 = (j & 1) | ((j >> 2) << 1), e = (j >> 1) & 1;
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = sm[(k1 * 32 + ((2 * m + e) ^ (k1 & 1))) * PS + p];
    dft16<INV>(v);
    // the e = 1 lane of a pair: W32^k' A_1[k'] (tw[0] = 1 exactly for e = 0)
#pragma unroll
    for (int k = 1; k < 16; ++k) {
      const C w = __ldg(&tw[16 * k * e]);
      v[k] = INV ? cmulc(v[k], w) : cmul(v[k], w);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      // e = 0: keeps A_0[i], sends A_0[8 + i], gets W A_1[i];
      // e = 1: keeps W A_1[8 + i], sends W A_1[i], gets A_0[8 + i]
      const C snd = e ? v[i] : v[8 + i];
      C rcv;
      rcv.x = __shfl_xor_sync(0xffffffffu, snd.x, 2 * P);
      rcv.y = __shfl_xor_sync(0xffffffffu, snd.y, 2 * P);
      const C a0 = e ? rcv : v[i];
      const C b = e ? v[8 + i] : rcv;
      const int kp = 8 * e + i;
      sm[(k1 + 16 * kp) * PS + p] = cadd(a0, b);
      sm[(k1 + 16 * (kp + 16)) * PS + p] = csub(a0, b);
    }
    __syncthreads();
  }

  template <bool INV>
  __device__ static void inplace_512(C* sm, const C* __restrict__ tw) {
    const int t = threadIdx.x;
    const int p = t % P, j = t / P;
    C v[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = sm[(j + S1 * m) * PS + p];
    phase1_512<INV>(v, tw);
    __syncthreads();
    finish_512<INV>(v, sm, tw);
  }

  // Input and output in shared memory, natural order, in place.  Ends with a
  // barrier.
  template <bool INV>
  __device__ static void run_inplace(C* sm, const C* __restrict__ tw) {
#ifndef SC_NO_TWO_PASS
    if constexpr (TWO_PASS) {
      inplace_512<INV>(sm, tw);
      return;
    }
#endif
    all_stages<0, INV>(sm, tw);
  }

  // Full transform: registers (first-stage layout) -> registers (last-stage
  // layout).  Ends with a barrier, so the caller may reuse `sm` at once.
  template <bool INV>
  __device__ static void run(C (&in)[J1][R1], C (&out)[JL][RL], C* sm, const C* __restrict__ tw) {
    if constexpr (NS == 1) {
#pragma unroll
      for (int a = 0; a < J1; ++a) {
#pragma unroll
        for (int r = 0; r < R1; ++r) out[a][r] = in[a][r];
        dft<R1, INV>(out[a]);
      }
    } else {
      // stage 0: registers -> shared (Ns = 1, no twiddles)
#pragma unroll
      for (int a = 0; a < J1; ++a) {
        int job = threadIdx.x + a * NT, p, j;
        decode<R1>(job, p, j);
        if ((TOT1 % NT == 0) || job < TOT1) {
          dft<R1, INV>(in[a]);
          store_stage0<R1>(in[a], sm, j, p);
        }
      }
      __syncthreads();
      mid_stages<1, INV>(sm, tw);
      last_stage<INV>(out, sm, tw);
    }
  }
};

}  // namespace sc
