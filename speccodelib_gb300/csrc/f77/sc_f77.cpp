// Fortran-callable shims with the reference's subroutine signatures
// (include/specns_f77.h), forwarding to the C ABI of libspecns.so.
// Built twice: -DSC_F77_SP (REAL = float) and -DSC_F77_DP (REAL = double).
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "specns.h"
#include "specns_f77.h"

namespace {

#ifdef SC_F77_SP
constexpr int kPrec = SC_FP32;
#else
constexpr int kPrec = SC_FP64;
#endif

// The reference's subroutines have no status argument, and its programs stop
// on a fatal state; by default a failing shim does the same (message, then
// abort).  specns_f77_set_abort(0) makes failures recoverable instead: the
// shim records the status and returns at once (its output arrays are then
// undefined), and specns_f77_status reports it.
bool g_abort = true;
int g_status = SC_OK;

bool check(int rc, const char* where) {
  if (rc == SC_OK) return true;
  if (g_abort) {
    std::fprintf(stderr, "specns %s: %s\n", where, sc_last_error());
    std::abort();
  }
  if (g_status == SC_OK) g_status = rc;
  return false;
}

int wave(int i, int n) { return i < n / 2 ? i : i - n; }

}  // namespace

#define SC_F77_CHECK(expr, where) \
  do {                            \
    if (!check((expr), where)) return; \
  } while (0)

extern "C" {

void convec_dns_(const void* vx, const void* vy, const void* vz, void* wx, void* wy, void* wz,
                 const int* lx1, const int* ly, const int* lz, const int* nx, const int* ny,
                 const int* nz) {
  SC_F77_CHECK(sc_convec_dns(kPrec, vx, vy, vz, wx, wy, wz, *lx1, *ly, *lz, *nx, *ny, *nz), "convec_dns");
}

void force_(void* wx, void* wy, void* wz, const void* vx, const void* vy, const void* vz,
            const sc_f77_real*, const int* lx1, const int* ly, const int* lz,
            const sc_f77_real* fkmax, const sc_f77_real* eps) {
  SC_F77_CHECK(sc_force(kPrec, wx, wy, wz, vx, vy, vz, *lx1, *ly, *lz, (double)*fkmax, (double)*eps), "force");
}

void force_rot_(void* wx, void* wy, void* wz, const void* vx, const void* vy, const void* vz,
                const sc_f77_real*, const int* lx1, const int* ly, const int* lz, const sc_f77_real* fk12,
                const sc_f77_real* fk22, const sc_f77_real* eps) {
  SC_F77_CHECK(sc_force_rot(kPrec, wx, wy, wz, vx, vy, vz, *lx1, *ly, *lz, (double)*fk12, (double)*fk22, (double)*eps),
        "force_rot");
}

void forcephi_(const void* phi, void* wphi, const sc_f77_real*, const int* lx1, const int* ly, const int* lz,
               const sc_f77_real* fkmax, const sc_f77_real* epsphi) {
  SC_F77_CHECK(sc_forcephi(kPrec, phi, wphi, *lx1, *ly, *lz, (double)*fkmax, (double)*epsphi), "forcephi");
}

void forcephi_rot_(const void* phi, void* wphi, const sc_f77_real*, const int* lx1, const int* ly, const int* lz,
                   const sc_f77_real* fk1, const sc_f77_real* fk2, const sc_f77_real* epsphi) {
  SC_F77_CHECK(sc_forcephi_rot(kPrec, phi, wphi, *lx1, *ly, *lz, (double)*fk1, (double)*fk2, (double)*epsphi),
        "forcephi_rot");
}

void convecphi_dns_(const void* vx, const void* vy, const void* vz, const void* phi, void* wphi,
                    const sc_f77_real*, const sc_f77_real*, const sc_f77_real*, const int* lx1, const int* ly,
                    const int* lz, const int* nx, const int* ny, const int* nz) {
  SC_F77_CHECK(sc_convecphi_dns(kPrec, vx, vy, vz, phi, wphi, *lx1, *ly, *lz, *nx, *ny, *nz), "convecphi_dns");
}

void skewness_(const void* ux, const sc_f77_real*, sc_f77_real* s, const int* nx, const int* ny, const int* nz) {
  double v = 0.0;
  SC_F77_CHECK(sc_skewness(kPrec, ux, *nx, *ny, *nz, &v), "skewness");
  *s = (sc_f77_real)v;
}

void enstrophy_(const void* ux, const void* uy, const void* uz, const double*, const double*, const double*,
                double* enstr, const int* lx1, const int* ly, const int* lz, const int*, const int* nx,
                const int* ny, const int* nz) {
  SC_F77_CHECK(sc_enstrophy(SC_FP64, ux, uy, uz, enstr, *lx1, *ly, *lz, *nx, *ny, *nz), "enstrophy");
}

void projection_(void* vx, void* vy, void* vz, const sc_f77_real*, const sc_f77_real*,
                 const sc_f77_real*, const int* lx1, const int* ly, const int* lz) {
  SC_F77_CHECK(sc_projection(kPrec, vx, vy, vz, *lx1, *ly, *lz), "projection");
}

void __msymmetrize_MOD_symmetrize3d(void* c, const int* lx1, const int* ly, const int* lz) {
  SC_F77_CHECK(sc_symmetrize(kPrec, c, *lx1, *ly, *lz), "symmetrize");
}

void symmetrize3d_(void* c, const int* lx1, const int* ly, const int* lz) {
  SC_F77_CHECK(sc_symmetrize(kPrec, c, *lx1, *ly, *lz), "symmetrize");
}

void hermitianize_(void* c, const int* lx1, const int* ly, const int* lz) {
  SC_F77_CHECK(sc_hermitianize(kPrec, c, *lx1, *ly, *lz), "hermitianize");
}

void dealiasing_(void* c, const sc_f77_real*, const int* lx1, const int* ly, const int* lz) {
  SC_F77_CHECK(sc_dealiasing(kPrec, c, *lx1, *ly, *lz), "dealiasing");
}

void smag_(const void* vx, const void* vy, const void* vz, void* t11, void* t12, void* t13,
           void* t22, void* t23, void* t33, const sc_f77_real*, const sc_f77_real*,
           const sc_f77_real*, const int* lx1, const int* ly, const int* lz, const int* nx,
           const int* ny, const int* nz, const sc_f77_real* delta) {
  SC_F77_CHECK(sc_smag(kPrec, vx, vy, vz, t11, t12, t13, t22, t23, t33, *lx1, *ly, *lz, *nx, *ny, *nz,
                (double)*delta, 0.026),
        "smag");
}

void dynsmag_(const void* ux, const void* uy, const void* uz, void* t11, void* t12, void* t13,
              void* t22, void* t23, void* t33, const sc_f77_real*, const sc_f77_real*,
              const sc_f77_real*, const sc_f77_real* g_test, const int* lx1, const int* ly,
              const int* lz, const int* nx, const int* ny, const int* nz, const int*,
              const sc_f77_real* delta, const sc_f77_real* delta_test, sc_f77_real* mm,
              sc_f77_real* lm, sc_f77_real* cs2, const int* update) {
  // Recover k_test from the sharp filter: the largest k2 it passes.
  long long k2in = -1, k2out = 1LL << 62;
  for (int kk = 0; kk < *lz; ++kk)
    for (int jj = 0; jj < *ly; ++jj)
      for (int ii = 0; ii < *lx1; ++ii) {
        const long long kz = wave(kk, *lz), ky = wave(jj, *ly);
        const long long k2 = (long long)ii * ii + ky * ky + kz * kz;
        const sc_f77_real gv = g_test[((long long)kk * *ly + jj) * *lx1 + ii];
        if (gv != 0) { if (k2 > k2in) k2in = k2; }
        else if (k2 < k2out) k2out = k2;
      }
  if (k2in >= k2out) {
    if (g_abort) {
      std::fprintf(stderr, "specns dynsmag: g_test is not a sharp spherical filter\n");
      std::abort();
    }
    if (g_status == SC_OK) g_status = SC_ERR_INVALID;
    return;
  }
  const double k_test = std::sqrt((double)k2in + 0.5);
  double dmm = 0, dlm = 0, dcs2 = (double)*cs2;
  SC_F77_CHECK(sc_dynsmag(kPrec, ux, uy, uz, t11, t12, t13, t22, t23, t33, *lx1, *ly, *lz, *nx, *ny, *nz,
                   k_test, (double)*delta, (double)*delta_test, &dmm, &dlm, &dcs2, *update != 0),
        "dynsmag");
  if (*update) {
    *mm = (sc_f77_real)dmm;
    *lm = (sc_f77_real)dlm;
    *cs2 = (sc_f77_real)dcs2;
  }
}

void specns_f77_set_abort_(const int* on) { g_abort = *on != 0; }

void specns_f77_status_(int* status) {
  *status = g_status;
  g_status = SC_OK;
}

}  // extern "C"
