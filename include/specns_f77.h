/*
 * specns_f77.h -- Fortran-callable drop-in entry points with the reference's
 * exact subroutine signatures (gfortran f77 ABI: lower-case name + '_', every
 * argument by reference, explicit-shape arrays as base pointers, LOGICAL as a
 * 4-byte integer, no hidden length arguments).
 *
 * Two libraries export them: libspecns_f77_dp.so (REAL = double,
 * complex(sp) = complex(8), the reference built with constant.f90) and
 * libspecns_f77_sp.so (REAL = float, the reference built with
 * constant_sp.f90).  Arrays are host memory; each call copies to the GPU,
 * runs the CUDA passes of libspecns.so and copies back.  On error the shim
 * prints sc_last_error() and aborts by default (the reference has no status
 * returns and its programs stop on fatal states); a caller that wants to
 * recover turns that off with specns_f77_set_abort_ and reads
 * specns_f77_status_ after its calls.
 */
#ifndef SPECNS_F77_H
#define SPECNS_F77_H

#ifdef SC_F77_SP
typedef float sc_f77_real;
#else
typedef double sc_f77_real;
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* convec_dns.f90:1 */
void convec_dns_(const void* vx, const void* vy, const void* vz, void* wx, void* wy, void* wz,
                 const int* lx1, const int* ly, const int* lz, const int* nx, const int* ny,
                 const int* nz);

/* force.f90:3 (k2 is accepted and ignored: the wavenumbers follow from the grid) */
void force_(void* wx, void* wy, void* wz, const void* vx, const void* vy, const void* vz,
            const sc_f77_real* k2, const int* lx1, const int* ly, const int* lz,
            const sc_f77_real* fkmax, const sc_f77_real* eps);

/* force_rot.f90:3 (k2 accepted and ignored; fk12, fk22 squared band bounds) */
void force_rot_(void* wx, void* wy, void* wz, const void* vx, const void* vy, const void* vz,
                const sc_f77_real* k2, const int* lx1, const int* ly, const int* lz,
                const sc_f77_real* fk12, const sc_f77_real* fk22, const sc_f77_real* eps);

/* forcephi.f90:1 (k2 accepted and ignored) */
void forcephi_(const void* phi, void* wphi, const sc_f77_real* k2, const int* lx1, const int* ly, const int* lz,
               const sc_f77_real* fkmax, const sc_f77_real* epsphi);

/* forcephi_rot.f90:1 (k2 accepted and ignored) */
void forcephi_rot_(const void* phi, void* wphi, const sc_f77_real* k2, const int* lx1, const int* ly, const int* lz,
                   const sc_f77_real* fk1, const sc_f77_real* fk2, const sc_f77_real* epsphi);

/* convecphi_dns.f90:1 (kx, ky, kz accepted and ignored) */
void convecphi_dns_(const void* vx, const void* vy, const void* vz, const void* phi, void* wphi,
                    const sc_f77_real* kx, const sc_f77_real* ky, const sc_f77_real* kz,
                    const int* lx1, const int* ly, const int* lz, const int* nx, const int* ny,
                    const int* nz);

/* skewness.f90:1 (kx accepted and ignored; s is real(sp)) */
void skewness_(const void* ux, const sc_f77_real* kx, sc_f77_real* s, const int* nx, const int* ny,
               const int* nz);

/* enstrophy.f90:1 (double precision in both builds, as the reference declares
 * it; kx, ky, kz accepted and ignored) */
void enstrophy_(const void* ux, const void* uy, const void* uz, const double* kx, const double* ky,
                const double* kz, double* enstr, const int* lx1, const int* ly, const int* lz, const int* lx,
                const int* nx, const int* ny, const int* nz);

/* projection.f90:2 (kx, ky, kz accepted and ignored) */
void projection_(void* vx, void* vy, void* vz, const sc_f77_real* kx, const sc_f77_real* ky,
                 const sc_f77_real* kz, const int* lx1, const int* ly, const int* lz);

/* symmetrize.f90:32 -- module procedure msymmetrize::symmetrize3d; exported
 * under gfortran's module mangling and under a plain f77 name */
void __msymmetrize_MOD_symmetrize3d(void* c, const int* lx1, const int* ly, const int* lz);
void symmetrize3d_(void* c, const int* lx1, const int* ly, const int* lz);

/* hermitianize.f90:1 */
void hermitianize_(void* c, const int* lx1, const int* ly, const int* lz);

/* dealiasing.f90:2 (k2 accepted and ignored) */
void dealiasing_(void* c, const sc_f77_real* k2, const int* lx1, const int* ly, const int* lz);

/* smag.f90:1 (c1 = 0.026 as in smag.f90:7) */
void smag_(const void* vx, const void* vy, const void* vz, void* t11, void* t12, void* t13,
           void* t22, void* t23, void* t33, const sc_f77_real* kx, const sc_f77_real* ky,
           const sc_f77_real* kz, const int* lx1, const int* ly, const int* lz, const int* nx,
           const int* ny, const int* nz, const sc_f77_real* delta);

/* dynsmag.f90:1 -- g_test must be the sharp filter [k2 <= k_test^2] of
 * spectral_les.f90:105-109; the shim recovers k_test from it. */
void dynsmag_(const void* ux, const void* uy, const void* uz, void* t11, void* t12, void* t13,
              void* t22, void* t23, void* t33, const sc_f77_real* kx, const sc_f77_real* ky,
              const sc_f77_real* kz, const sc_f77_real* g_test, const int* lx1, const int* ly,
              const int* lz, const int* nx, const int* ny, const int* nz, const int* lx,
              const sc_f77_real* delta, const sc_f77_real* delta_test, sc_f77_real* mm,
              sc_f77_real* lm, sc_f77_real* cs2, const int* update);

/* No reference counterpart.  on = 0: a failing shim records its status
 * (SC_ERR_*) and returns at once, its output arrays undefined; on = 1 (the
 * default): it prints sc_last_error() and aborts.  Fortran:
 * call specns_f77_set_abort(0). */
void specns_f77_set_abort_(const int* on);

/* No reference counterpart.  The status of the first failure since the
 * previous query (SC_OK if none), then cleared. */
void specns_f77_status_(int* status);

#ifdef __cplusplus
}
#endif
#endif /* SPECNS_F77_H */
