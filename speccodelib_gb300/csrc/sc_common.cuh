// Common device types and helpers for the spectral Navier-Stokes kernels.
//
// Field layout in HBM (internal, all kernels): a half-complex field is
// (nz, ny, nxp) complex in C order, row pitch nxp >= nx/2+1 a multiple of the
// pencil tile width, so every row starts on a 128-byte boundary.  Element
// (kz|z, ky|y, kx) lives at (z*ny + y)*nxp + kx.  Columns kx >= nx/2+1 are
// padding: zero-filled at allocation, never read by a transform and never
// written with non-zero data.  The reference's Fortran array c(lx1,ly,lz) is
// the same ordering with pitch lx1 = nx/2+1; host<->device copies repack
// between the two pitches with a 2D memcpy.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sc {

template <typename T> struct V2;
template <> struct V2<float> { using t = float2; };
template <> struct V2<double> { using t = double2; };

template <typename T> using C2 = typename V2<T>::t;

template <typename C> __device__ __forceinline__ C mk(decltype(C::x) a, decltype(C::x) b) {
  C r; r.x = a; r.y = b; return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
  return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {
  return mk<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C> __device__ __forceinline__ C cconj(C a) { return mk<C>(a.x, -a.y); }
// i * a
template <typename C> __device__ __forceinline__ C cmuli(C a) { return mk<C>(-a.y, a.x); }
// -i * a
template <typename C> __device__ __forceinline__ C cmulmi(C a) { return mk<C>(a.y, -a.x); }
template <typename C, typename R> __device__ __forceinline__ C cscale(C a, R s) { return mk<C>(a.x * s, a.y * s); }
template <typename C> __device__ __forceinline__ C czero() { return mk<C>(0, 0); }

#ifndef SC_NO_F32X2
// FP32 complex add, subtract and real scale as single packed sm_100-family
// instructions (add/sub/mul.rn.f32x2): each component is rounded exactly as
// the scalar form, but the butterflies issue half the instructions.
__device__ __forceinline__ unsigned long long f2_pack(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
template <> __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(d);
}
template <> __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(d);
}
template <> __device__ __forceinline__ float2 cscale<float2, float>(float2 a, float s) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_pack(a)), "l"(f2_pack(make_float2(s, s))));
  return f2_unpack(d);
}
#endif

// Signed wavenumber of index i on an axis of length n: 0..n/2-1, -n/2..-1
// (the FFTW ordering, wavenumber.f90:109,115).
__device__ __forceinline__ int wavenum(int i, int n) { return i < n / 2 ? i : i - n; }

// Integer forms of a real bound t on an integer k^2 (exact in int: 3 (n/2)^2
// < 2^31 for every supported n):  k2 < t  <=>  k2 < k2_lt(t),  and
// k2 <= t  <=>  k2 < k2_le(t).  Computed once per kernel, they keep the
// per-point wavenumber tests in integer arithmetic (double-precision
// throughput on this part is a small fraction of single precision).
__host__ __device__ inline int k2_clamp(double b) {
  return b >= 2147483647.0 ? 2147483647 : (b <= -2147483647.0 ? -2147483647 : (int)b);
}
__host__ __device__ inline int k2_lt(double t) { return k2_clamp(ceil(t)); }

// floor(sqrt(k2) + 1/2) for an integer k2 >= 0, exactly: the n with
// n^2 - n < k2 <= n^2 + n (a float root is within one of it).
__host__ __device__ __forceinline__ int shell_index(int k2) {
  int n = (int)(sqrtf((float)k2) + 0.5f);
  const long long nn = (long long)n * n;
  if (nn + n < k2) ++n;
  else if (n > 0 && nn - n >= k2) --n;
  return n;
}

// Grid-stride walk over the points (ix, iy, iz) of an index space of n x ny
// x (any) points, ix fastest, from point t0 in steps of `stride` points: the
// coordinates are carried from step to step (two 64-bit divisions per thread
// instead of three per point).
struct Walk3 {
  long long t, total, stride;
  int ix, iy, iz;
  int n, ny, dix, diy, diz;
  __host__ __device__ __forceinline__ Walk3(long long t0, long long stride_, long long total_, int n_, int ny_)
      : t(t0), total(total_), stride(stride_), n(n_), ny(ny_) {
    const long long r = t0 / n_, sr = stride_ / n_;
    ix = (int)(t0 - r * n_);
    iy = (int)(r % ny_);
    iz = (int)(r / ny_);
    dix = (int)(stride_ - sr * n_);
    diy = (int)(sr % ny_);
    diz = (int)(sr / ny_);
  }
  __host__ __device__ __forceinline__ bool ok() const { return t < total; }
  __host__ __device__ __forceinline__ void next() {
    t += stride;
    ix += dix;
    int c = ix >= n;
    if (c) ix -= n;
    iy += diy + c;
    c = iy >= ny;
    if (c) iy -= ny;
    iz += diz + c;
  }
  __host__ __device__ __forceinline__ long long row() const { return (long long)iz * ny + iy; }
};
__host__ __device__ inline int k2_le(double t) { return k2_clamp(floor(t) + 1.0); }

// Grid geometry shared by all passes.
struct Geom {
  int nx, ny, nz;      // physical grid
  int nxh;             // nx/2 + 1 complex columns
  int nxp;             // padded row pitch (complex elements)
  long long field;     // elements per field = nz*ny*nxp
};

constexpr int kMaxFields = 18;

template <typename T> struct FieldList {
  C2<T>* f[kMaxFields];
};

}  // namespace sc
