/*
 * Oracle (test infrastructure only): seeded Gaussian spectral fields.
 *
 * CPU restatement of the reference's random-phase generator so the oracle can
 * reproduce its seeded initial fields mode for mode:
 *   ran1   -- initialize.f90:516-548 (Numerical Recipes "ran1": Park-Miller
 *             minimal standard generator, Schrage factorisation, 32-entry
 *             Bays-Durham shuffle table, 8 warm-up draws).
 *   gasdev -- initialize.f90:507-513 (complex Box-Muller draw divided by
 *             sqrt(2) so the complex variance is 1).
 *   loop   -- initialize.f90:305-326: modes visited kk (z) outer, jj (y),
 *             ii (x) inner; per mode and component two draws (t1, t2) with
 *             t2 <- 2*pi*t2 and pi = 3.1415926536 (constant_sp.f90:20).
 * The double-precision ("-dp") build of the reference is followed: am, eps and
 * the Box-Muller arithmetic are in double.
 *
 * Only tests, smoke() and the CPU-baseline leg of bench.py may use this file.
 */
#include <math.h>
#include <stdint.h>

#define RAN1_IA 16807
#define RAN1_IM 2147483647
#define RAN1_IQ 127773
#define RAN1_IR 2836
#define RAN1_NTAB 32
#define RAN1_NDIV (1 + (RAN1_IM - 1) / RAN1_NTAB)

typedef struct {
  int32_t idum;
  int32_t iy;
  int32_t iv[RAN1_NTAB];
} oracle_ran1_state;

static int32_t park_miller(int32_t idum) {
  int32_t k = idum / RAN1_IQ;
  idum = RAN1_IA * (idum - k * RAN1_IQ) - RAN1_IR * k;
  if (idum < 0) idum += RAN1_IM;
  return idum;
}

static double oracle_ran1(oracle_ran1_state *s) {
  const double am = 1.0 / (double)RAN1_IM;
  const double rnmx = 1.0 - 1.2e-7;
  if (s->idum <= 0 || s->iy == 0) {
    /* idum = max(-idum, 1): every positive seed restarts the stream of 1 */
    int32_t idum = -s->idum;
    if (idum < 1) idum = 1;
    for (int j = RAN1_NTAB + 8; j >= 1; --j) {
      idum = park_miller(idum);
      if (j <= RAN1_NTAB) s->iv[j - 1] = idum;
    }
    s->iy = s->iv[0];
    s->idum = idum;
  }
  s->idum = park_miller(s->idum);
  int j = s->iy / RAN1_NDIV; /* 0-based slot of 1 + iy/ndiv */
  s->iy = s->iv[j];
  s->iv[j] = s->idum;
  double r = am * (double)s->iy;
  return r < rnmx ? r : rnmx;
}

/* The generator's integer state idum after `ncalls` calls of ran1 from a
 * fresh generator seeded with `seed` (the warm-up's 8 + 32 Park-Miller steps
 * run in the first call).  Each call advances idum by exactly one
 * Park-Miller step, so from seed 1 the state after 9960 calls is z_10000 of
 * the minimal standard sequence started at z_0 = 1. */
int32_t oracle_ran1_state_after(int32_t seed, int64_t ncalls) {
  oracle_ran1_state s = {0};
  s.idum = seed;
  for (int64_t i = 0; i < ncalls; ++i) (void)oracle_ran1(&s);
  return s.idum;
}

/* z_n of the bare Park-Miller minimal standard generator from z_0 = z0
 * (Schrage's factorisation, the same step ran1 uses). */
int32_t oracle_park_miller_after(int32_t z0, int64_t n) {
  int32_t z = z0;
  for (int64_t i = 0; i < n; ++i) z = park_miller(z);
  return z;
}

/* First `count` ran1 values for a fresh generator seeded with `seed`. */
void oracle_ran1_sequence(int32_t seed, int64_t count, double *out) {
  oracle_ran1_state s = {0};
  s.idum = seed;
  for (int64_t i = 0; i < count; ++i) out[i] = oracle_ran1(&s);
}

/*
 * Draw `ncomp` complex Gaussian fields of shape (nz, ny, nxh) (C order, i.e.
 * Fortran (nxh, ny, nz)); out holds ncomp consecutive fields as interleaved
 * (re, im) doubles.  Component c of mode (kk, jj, ii) uses draws
 * 6*mode + 2c, 6*mode + 2c + 1 when ncomp = 3.
 */
void oracle_gauss_fields(int nxh, int ny, int nz, int ncomp, int32_t seed,
                         double *out) {
  const double pi_ref = 3.1415926536;
  const int64_t plane = (int64_t)nxh * ny * nz;
  oracle_ran1_state s = {0};
  s.idum = seed;
  for (int kk = 0; kk < nz; ++kk)
    for (int jj = 0; jj < ny; ++jj)
      for (int ii = 0; ii < nxh; ++ii) {
        int64_t idx = ((int64_t)kk * ny + jj) * nxh + ii;
        for (int c = 0; c < ncomp; ++c) {
          double t1 = oracle_ran1(&s);
          double t2 = oracle_ran1(&s);
          t2 = 2.0 * pi_ref * t2;
          double a = sqrt(-2.0 * log(t1));
          out[2 * (c * plane + idx) + 0] = a * cos(t2) / sqrt(2.0);
          out[2 * (c * plane + idx) + 1] = a * sin(t2) / sqrt(2.0);
        }
      }
}
