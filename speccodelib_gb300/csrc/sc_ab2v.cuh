// Variable-step integrating-factor AB2 of spectral_dns.f90 / spectral_les.f90,
// per mode.
//
// The solvers choose each step dt from a CFL estimate and the next output
// time (spectral_dns.f90:212-217) and advance v with exp(-nu k^2 dt):
//   pass 0:   v = (v + dt w) e(dt); the initial field and w are kept (:220-228)
//   pass 1:   v = (S v0 e(dto) + ek v + delta w) e(dt) with r = dt/dto,
//             S = (1 + r^2)/2, ek = (1 - r^2)/2, delta = dto (1 + r)^2 / 2:
//             a restart from the initial field over dto + dt (:230-250)
//   pass >= 2: v = (v + S w + ek o e(dto)) e(dt) with S = (1 + r/2) dt,
//             ek = -(r/2) dt and o the previous right-hand side (:252-275)
// then v = 0 at k^2 >= kcut^2 and at the mean mode (:281-290).  The weights
// depend on the pass only (ab2v_weights, on the host); e(.) is evaluated per
// mode.
#pragma once
#include "sc_cx.cuh"

namespace sc {

// The weights (s, ek, dl) of a pass with step dt after the previous step dto
// (spectral_dns.f90:231-235 for pass 1, :253-257 for later passes; pass 0
// has none).
__host__ __device__ inline void ab2v_weights(int pass, double dt, double dto, double& s, double& ek, double& dl) {
  s = ek = dl = 0.0;
  if (pass < 1) return;
  const double r = dt / dto;
  if (pass == 1) {
    s = 0.5 * (1.0 + r * r);
    ek = 0.5 * (1.0 - r * r);
    dl = 0.5 * dto * (1.0 + r) * (1.0 + r);
  } else {
    s = (1.0 + 0.5 * r) * dt;
    ek = -0.5 * r * dt;
  }
}

// One pass at one mode of squared wavenumber k2.
//   pass 0: reads v; writes v0 = v, o = w and v
//   pass 1: reads v, v0; writes v
//   pass >= 2: reads v, o; writes o = w and v
// zero: the mode is cut (k^2 >= kcut^2) or the mean mode.
template <typename T>
__host__ __device__ inline void ab2v_point(int pass, int k2, bool zero, T nu, T dt, T dto, T s, T ek, T dl,
                                           Cx<T> v[3], const Cx<T> w[3], Cx<T> o[3], Cx<T> v0[3]) {
  const T e1 = exp(-(T)k2 * nu * dt);
  if (pass == 0) {
    for (int c = 0; c < 3; ++c) {
      v0[c] = v[c];
      o[c] = w[c];
      v[c] = cx_scale(cx_add(v[c], cx_scale(w[c], dt)), e1);                             // :222-224
    }
  } else {
    const T e0 = exp(-(T)k2 * nu * dto);
    for (int c = 0; c < 3; ++c) {
      Cx<T> vn;
      if (pass == 1)                                                                        // :239-246
        vn = cx_add(cx_add(cx_scale(cx_scale(v0[c], s), e0), cx_scale(v[c], ek)), cx_scale(w[c], dl));
      else                                                                                  // :259-268
        vn = cx_add(cx_add(v[c], cx_scale(w[c], s)), cx_scale(cx_scale(o[c], ek), e0));
      v[c] = cx_scale(vn, e1);
      if (pass >= 2) o[c] = w[c];                                                           // :270-272
    }
  }
  if (zero)
    for (int c = 0; c < 3; ++c) v[c] = cx(T(0), T(0));
}

// The passive scalar of spectral_dns_scalar.f90 on the same passes, with
// exp(-nu k2 dt / pr) (:267-329).  The history saved at pass 0 is phi after
// its update when hist_rhs is false, as written (outputphi(phi, 0), :278,
// read back at :308), else wphi (the evident intent).
//   pass 0: phi0 = phi, phi = (phi + dt wphi) e(dt), ophi = phi or wphi
//   pass 1: phi = (S phi0 e(dto) + ek phi + delta wphi) e(dt)
//   pass >= 2: phi = (phi + S wphi + ek ophi e(dto)) e(dt), ophi = wphi
template <typename T>
__host__ __device__ inline void ab2v_scalar_point(int pass, int k2, bool hist_rhs, T nu, T dt, T dto, T pr, T s, T ek,
                                                  T dl, Cx<T>& phi, Cx<T> wphi, Cx<T>& ophi, Cx<T>& phi0) {
  const T e1 = exp(-(T)k2 * nu * dt / pr);
  if (pass == 0) {
    phi0 = phi;
    phi = cx_scale(cx_add(phi, cx_scale(wphi, dt)), e1);                                   // :273
    ophi = hist_rhs ? wphi : phi;
    return;
  }
  const T e0 = exp(-(T)k2 * nu * dto / pr);
  Cx<T> pn;
  if (pass == 1)                                                                            // :295
    pn = cx_add(cx_add(cx_scale(cx_scale(phi0, s), e0), cx_scale(phi, ek)), cx_scale(wphi, dl));
  else                                                                                      // :321
    pn = cx_add(cx_add(phi, cx_scale(wphi, s)), cx_scale(cx_scale(ophi, ek), e0));
  phi = cx_scale(pn, e1);                                                                   // :303, :329
  if (pass >= 2) ophi = wphi;                                                               // :335
}

}  // namespace sc
