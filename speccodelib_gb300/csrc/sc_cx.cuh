// Complex arithmetic on plain scalars for the per-mode stepper updates
// (sc_rot.cuh, sc_ab2v.cuh): marked __host__ __device__ so that the same
// update code runs in the kernels and in host-side checks against the oracle.
#pragma once
#include <math.h>

namespace sc {

template <typename T> struct Cx { T re, im; };

template <typename T> __host__ __device__ inline Cx<T> cx(T re, T im) { Cx<T> r; r.re = re; r.im = im; return r; }
template <typename T> __host__ __device__ inline Cx<T> cx_add(Cx<T> a, Cx<T> b) { return cx(a.re + b.re, a.im + b.im); }
template <typename T> __host__ __device__ inline Cx<T> cx_sub(Cx<T> a, Cx<T> b) { return cx(a.re - b.re, a.im - b.im); }
template <typename T> __host__ __device__ inline Cx<T> cx_mul(Cx<T> a, Cx<T> b) {
  return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
// a * conj(b)
template <typename T> __host__ __device__ inline Cx<T> cx_mulc(Cx<T> a, Cx<T> b) {
  return cx(a.re * b.re + a.im * b.im, a.im * b.re - a.re * b.im);
}
template <typename T> __host__ __device__ inline Cx<T> cx_scale(Cx<T> a, T s) { return cx(a.re * s, a.im * s); }
template <typename T> __host__ __device__ inline Cx<T> cx_conj(Cx<T> a) { return cx(a.re, -a.im); }

}  // namespace sc
