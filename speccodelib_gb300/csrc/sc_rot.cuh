// Helical-wave integrating-factor AB2 of the rotating solver, per mode.
//
// spectral_rot_dns_ft.f90 keeps the velocity as two helical amplitudes,
// a+ = v . conj(h) and a- = v . h (:132-133), with h the positive-helicity
// unit vector of heliwave.f90:57-96 (i k x h = |k| h).  Each amplitude is
// advanced with its own complex integrating factor
//   ef+- = exp(-nu k^2 dt +- 2 i dt kz om / |k|)        (:101-111)
// (viscous decay and the inertial-wave phase of rotation rate om): pass 0 is
// an Euler half step (:215-223), pass 1 a midpoint restart from the initial
// field (:225-237), later passes AB2 with the previous right-hand side
// (:239-256); the velocity is rebuilt as a+ h + a- conj(h) and truncated at
// k^2 >= kcut^2 (:261-270).  The amplitudes themselves are never truncated.
//
// Everything here is plain scalar arithmetic marked __host__ __device__
// (sc_cx.cuh), so the same code runs in rot_update_kernel and in host-side
// checks.
#pragma once
#include "sc_cx.cuh"

namespace sc {

// h+ at integer wavenumber (kx, ky, kz), heliwave.f90:73-91.  Rows with
// ky = kz = 0 (:73-81) have k2d = max(|kx|, smallest) and reduce to
// h = (0, 1, i)/sqrt(2) for kx > 0 (every numerator of the mean mode is
// zero, so h = 0 there); the others (:82-91) have k2d = sqrt(ky^2 + kz^2) > 0.
template <typename T> __host__ __device__ inline void heli_vector(int kx, int ky, int kz, Cx<T> h[3]) {
  const T s = (T)0.70710678118654752440;   // sqrt(2)/2
  if (ky == 0 && kz == 0) {
    const T on = kx != 0 ? s : T(0);
    h[0] = cx(T(0), T(0));
    h[1] = cx(on, T(0));
    h[2] = cx(T(0), on);
    return;
  }
  const T fx = (T)kx, fy = (T)ky, fz = (T)kz;
  const T d2 = fy * fy + fz * fz;
  const T k = sqrt(fx * fx + d2), kd = sqrt(d2);
  const T rkd = T(1) / kd, rkk = T(1) / (k * kd);
  h[0] = cx(T(0), s * d2 * rkk);
  h[1] = cx(-s * fz * rkd, -s * fx * fy * rkk);
  h[2] = cx(s * fy * rkd, -s * fz * fx * rkk);
}

// ef = exp(-nu k2 dt + i ph) and its principal square root, ph =
// 2 dt kz om / |k| (0 at the mean mode, where the reference's
// kz / (sqrt(tiny) + tiny) is 0).  ef- = conj(ef+), sqrt(ef-) = conj(sqrt(ef+)).
template <typename T>
__host__ __device__ inline void rot_factor(int k2, int kz, T nu, T dt, T om, Cx<T>& ef, Cx<T>& sq) {
  const T pi = (T)3.14159265358979323846;
  T ph = k2 > 0 ? T(2) * dt * (T)kz * om / sqrt((T)k2) : T(0);
  if (ph > pi || ph < -pi) ph = remainder(ph, T(2) * pi);   // principal branch of the square root
  const T decay = -(T)k2 * nu * dt;
  const T mag = exp(decay), smag = exp(T(0.5) * decay);
  ef = cx(mag * cos(ph), mag * sin(ph));
  sq = cx(smag * cos(T(0.5) * ph), smag * sin(T(0.5) * ph));
}

// x . conj(h) and x . h
template <typename T> __host__ __device__ inline Cx<T> dot_conj(const Cx<T> x[3], const Cx<T> h[3]) {
  return cx_add(cx_add(cx_mulc(x[0], h[0]), cx_mulc(x[1], h[1])), cx_mulc(x[2], h[2]));
}
template <typename T> __host__ __device__ inline Cx<T> dot_plain(const Cx<T> x[3], const Cx<T> h[3]) {
  return cx_add(cx_add(cx_mul(x[0], h[0]), cx_mul(x[1], h[1])), cx_mul(x[2], h[2]));
}

// One pass of the helical AB2 at one mode.
//   pass 0: reads v (the initial field), writes a = (a+, a-) of v, o = w,
//           and v = the half-step field
//   pass 1: reads a (still the initial amplitudes), writes a and v
//   pass >= 2: reads a and o, writes a, o = w and v
// cut: the mode lies at k^2 >= kcut^2 (v is zeroed there, a is kept).
template <typename T>
__host__ __device__ inline void rot_point(int pass, int kx, int ky, int kz, bool cut, T nu, T dt, T om,
                                          Cx<T> v[3], const Cx<T> w[3], Cx<T> o[3], Cx<T>& ap, Cx<T>& am) {
  Cx<T> h[3];
  heli_vector<T>(kx, ky, kz, h);
  Cx<T> efp, sqp;
  rot_factor<T>(kx * kx + ky * ky + kz * kz, kz, nu, dt, om, efp, sqp);
  const Cx<T> efm = cx_conj(efp), sqm = cx_conj(sqp);
  const T dth = T(0.5) * dt;
  Cx<T> np_, nm_;   // amplitudes after the pass
  if (pass == 0) {
    ap = dot_conj(v, h);                                                // :132
    am = dot_plain(v, h);                                               // :133
    np_ = cx_mul(cx_add(ap, cx_scale(dot_conj(w, h), dth)), sqp);       // :216
    nm_ = cx_mul(cx_add(am, cx_scale(dot_plain(w, h), dth)), sqm);      // :217
    for (int c = 0; c < 3; ++c) o[c] = w[c];                            // :223, :235
  } else if (pass == 1) {
    np_ = cx_add(cx_mul(ap, efp), cx_mul(cx_scale(dot_conj(w, h), dt), sqp));    // :227-228
    nm_ = cx_add(cx_mul(am, efm), cx_mul(cx_scale(dot_plain(w, h), dt), sqm));   // :229
    ap = np_;
    am = nm_;
  } else {
    Cx<T> t[3];
    for (int c = 0; c < 3; ++c) t[c] = cx_sub(cx_scale(w[c], T(3)), cx_mul(efp, o[c]));   // :240-242
    np_ = cx_mul(cx_add(ap, cx_scale(dot_conj(t, h), dth)), efp);                        // :243
    for (int c = 0; c < 3; ++c) t[c] = cx_sub(cx_scale(w[c], T(3)), cx_mul(efm, o[c]));   // :245-247
    nm_ = cx_mul(cx_add(am, cx_scale(dot_plain(t, h), dth)), efm);                       // :248
    for (int c = 0; c < 3; ++c) o[c] = w[c];                                             // :250-252
    ap = np_;
    am = nm_;
  }
  for (int c = 0; c < 3; ++c)                                                           // :261-270
    v[c] = cut ? cx(T(0), T(0)) : cx_add(cx_mul(np_, h[c]), cx_mul(nm_, cx_conj(h[c])));
}

// The passive scalar of spectral_rot_dns_scalar_ft.f90 on the same pass
// schedule, with efphi = exp(-nu k2 dt / pr) (:104):
//   pass 0: phi0 = phi, ophi = wphi, phi = (phi + dt/2 wphi) sqrt(efphi)  (:230)
//   pass 1: phi = phi0 efphi + dt wphi sqrt(efphi)                       (:249)
//   pass >= 2: phi = (phi + dt/2 (3 wphi - ophi efphi)) efphi, ophi = wphi (:278-279)
template <typename T>
__host__ __device__ inline void rot_scalar_point(int pass, int k2, T nu, T dt, T pr, Cx<T>& phi, Cx<T> wphi,
                                                 Cx<T>& ophi, Cx<T>& phi0) {
  const T decay = -(T)k2 * nu * dt / pr;
  const T ef = exp(decay), sq = exp(T(0.5) * decay);
  const T dth = T(0.5) * dt;
  if (pass == 0) {
    phi0 = phi;
    ophi = wphi;
    phi = cx_scale(cx_add(phi, cx_scale(wphi, dth)), sq);
  } else if (pass == 1) {
    phi = cx_add(cx_scale(phi0, ef), cx_scale(cx_scale(wphi, dt), sq));
  } else {
    phi = cx_scale(cx_add(phi, cx_scale(cx_sub(cx_scale(wphi, T(3)), cx_scale(ophi, ef)), dth)), ef);
    ophi = wphi;
  }
}

}  // namespace sc
