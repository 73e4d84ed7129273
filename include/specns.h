/*
 * specns.h -- C ABI of the GB300-native pseudo-spectral Navier-Stokes step.
 *
 * Drop-in boundary for the hot path of yili-shef/SpecCodeLib: the right-hand
 * side of the incompressible Navier-Stokes equations in rotational form
 * (Lamb vector, forcing, symmetrize, projection, optional Smagorinsky /
 * dynamic-Smagorinsky stress) and its integrating-factor time steps, on one
 * GPU.  Arrays crossing this boundary use the reference's FFTW r2c
 * half-complex layout: a Fortran complex(sp) array c(nx/2+1, ny, nz),
 * kx fastest, spectral coefficients normalised as
 * u^ = (1/(nx ny nz)) sum_x u e^{-ik.x}.
 *
 * Every function returns an int status: SC_OK or one of SC_ERR_*; the text of
 * the last error on the calling thread is returned by sc_last_error().
 * A handle is used by one host thread at a time.  Host pointers may be
 * pageable or pinned; device pointers must be CUDA device memory.
 * Precision of element data follows sc_params.precision: SC_FP32 arrays are
 * complex(4) (two floats per element), SC_FP64 arrays complex(8).
 */
#ifndef SPECNS_H
#define SPECNS_H

#ifdef __cplusplus
extern "C" {
#endif

#define SC_OK 0
#define SC_ERR_INVALID 1     /* bad argument or unsupported size */
#define SC_ERR_CUDA 2        /* a CUDA call failed */
#define SC_ERR_NONFINITE 3   /* NaN/Inf found in the state */
#define SC_ERR_TIMEOUT 4     /* a bounded device wait gave up */
#define SC_ERR_NOMEM 5       /* device allocation failed */
#define SC_ERR_IO 6          /* a file could not be read or written, or its records do not match */

#define SC_FP32 0            /* FP32 bulk (twiddles rounded from FP64, FP64 reductions) */
#define SC_FP64 1            /* plain FP64 */

#define SC_SGS_NONE 0
#define SC_SGS_SMAG 1        /* smag.f90 */
#define SC_SGS_DYNSMAG 2     /* dynsmag.f90 */

#define SC_MASK_AFTER_STEP 0   /* 2/3 truncation of the state after each step (dns-deform.f90:233-237) */
#define SC_MASK_RHS_AND_STEP 1 /* also truncate every right-hand side */

typedef struct sc_params {
  int nx, ny, nz;        /* grid; each a power of two in [8, 1024] */
  int precision;         /* SC_FP32 | SC_FP64 */
  double nu;             /* kinematic viscosity */
  double dt;             /* time step */
  int forced;            /* constant-power forcing on/off (force.f90) */
  double eps;            /* injected power */
  double fkmax;          /* forcing band k2 < fkmax^2 */
  double kcut;           /* 2/3 cutoff; 0 -> 2*(nx/2)/3 (dns-deform.f90:75) */
  int sgs;               /* SC_SGS_* */
  double c1;             /* Smagorinsky c1 = Cs^2 (smag.f90:7 hard-codes 0.026) */
  double delta;          /* filter width; 0 -> pi/kcut (spectral_les.f90:87) */
  double delta_ratio;    /* test-filter width ratio; 0 -> 2 (spectral_les.f90:16) */
  int dyn_every;         /* dynamic coefficient refresh interval; 0 -> 10 */
  int mask_mode;         /* SC_MASK_* */
} sc_params;

typedef struct sc_diag {
  double energy;         /* sum of 1/2-weighted |v|^2 (specdns-forced-omp-ft.f90:142-144) */
  double enstrophy;      /* sum k^2 q(k) */
  double dissipation;    /* 2 nu sum k^2 q(k) (meaneps.f90:37-44, per mode) */
  double max_div;        /* max |k . v^| */
  double max_u;          /* max |u| over grid points (CFL) */
  double nonfinite;      /* count of non-finite values seen */
  double cs2;            /* current Smagorinsky coefficient (c1 or dynamic cs2) */
  double mm, lm;         /* last dynamic-procedure sums (dynsmag.f90:176,184) */
} sc_diag;

typedef struct sc_handle sc_handle;

/* defaults for an n^3 grid: the forced-DNS configuration nu=0.01, dt=2e-3,
 * eps=0.1, fkmax=2.5 (shells k<=2), 2/3 rule, no SGS. */
int sc_default_params(sc_params* p, int n, int precision);

/* Create / destroy a solver instance; allocates its device state.
 * Replaces fftwplan3d / destroyplan3d (fftwplan.f90:7-30) and the
 * program-level allocations (specdns-forced-omp-ft.f90:81-86). */
int sc_create(const sc_params* p, sc_handle** out);
int sc_destroy(sc_handle* h);

/* Make CUDA device `device` current for this library on the calling thread
 * (handles are created on the current device). */
int sc_set_device(int device);

/* Launch on this CUDA stream (cudaStream_t passed as void*; NULL = the
 * handle's own stream). */
int sc_set_stream(sc_handle* h, void* stream);
/* Change dt (recomputes the integrating-factor tables). */
int sc_set_dt(sc_handle* h, double dt);

/* The handle's parameters (after defaults were filled in at sc_create). */
int sc_get_params(sc_handle* h, sc_params* out);

/* State upload / download in the reference layout (host pointers).
 * Replaces input / output of input.f90:106-136, output.f90:103-132. */
int sc_set_state(sc_handle* h, const void* vx, const void* vy, const void* vz);
int sc_get_state(sc_handle* h, void* vx, void* vy, void* vz);
/* Same with device pointers (reference layout, pitch nx/2+1). */
int sc_set_state_device(sc_handle* h, const void* vx, const void* vy, const void* vz);
int sc_get_state_device(sc_handle* h, void* vx, void* vy, void* vz);

/* Seeded initial field: initialize3dvelhighmemdealiased (initialize.f90:
 * 284-371) with Numerical Recipes ran1/gasdev (initialize.f90:507-548) in the
 * reference's draw order.  kind 0: amplitude ~ k exp(-k^2/akp^2) (E(k) ~
 * k^4 exp(-2 (k/akp)^2)); kind 1: E(k) ~ k^(-5/3) on kmin <= |k| <= kmax.
 * Rescaled to energy 3/2 u0^2. */
int sc_init_field(sc_handle* h, int seed, int kind, double akp, double u0, double kmin,
                  double kmax);

/* Right-hand side of the current state: dns-deform.f90:259-288 (ratesdudt)
 * plus the SGS divergence of spectral_les.f90:232-234 when sgs != NONE.
 * Outputs are host arrays in the reference layout. */
int sc_rhs(sc_handle* h, void* wx, void* wy, void* wz);

/* nsteps integrating-factor RK4 steps of dns-deform.f90:160-237 (computed in
 * the equivalent division-free form). */
int sc_rk4_steps(sc_handle* h, int nsteps);
/* npasses passes of the IF-AB2 loop of specdns-forced-omp-ft.f90:224-287
 * (pass 0: Euler half step; pass 1: midpoint restart; then AB2).  Its RHS is
 * the AB2 solver's own: no symmetrize (specdns-forced-omp-ft.f90:180-221). */
int sc_ab2_steps(sc_handle* h, int npasses);

/* One pass of the variable-step IF-AB2 of spectral_dns.f90:173-290 (and of
 * spectral_les.f90:199-316 with an SGS handle) with step dt.  Pass 0: an
 * integrating-factor Euler step; pass 1: a restart from the initial field
 * over dto + dt with the weights of dt/dto; later passes: AB2 weighted by
 * dt/dto with the previous right-hand side.  Its RHS has no symmetrize
 * (spectral_dns.f90:173-208).  After each pass v = 0 at k >= kcut and at the
 * mean mode; spectral_dns.f90 cuts at k >= nx/2 (set kcut = nx/2),
 * spectral_les.f90 at its kcut.  A dynsmag handle refreshes its coefficient
 * on passes 0, 1, 11, 21, ... (spectral_les.f90:140,205-208).  The handle
 * keeps the pass count and dto (two extra groups of three fields);
 * sc_set_state and sc_init_field restart at pass 0. */
int sc_ab2v_pass(sc_handle* h, double dt);
/* One pass of spectral_dns_scalar.f90:222-342: the variable-step IF-AB2 of
 * sc_ab2v_pass carrying the passive scalar of sc_set_scalar.  Velocity RHS:
 * Lamb vector, force, symmetrize (its five-argument symmetrize(w, k2, ...)
 * read as symmetrize3d), projection; scalar RHS: convecphi_dns, minus
 * meangrad * v_z when scalarforced (:244-246), symmetrized; the scalar
 * advances with exp(-nu k^2 dt / pr); v is not truncated after the update.
 * history_rhs = 0 keeps the program as written: pass 0 saves phi after its
 * update as the scalar's history (outputphi(phi, 0), :278); 1 saves wphi.
 * Shares the pass count and dto of sc_ab2v_pass; sc_set_scalar restarts. */
int sc_ab2v_scalar_pass(sc_handle* h, double dt, double pr, int scalarforced, double meangrad, int history_rhs);
/* The variable-step AB2's pass count and previous step dto (0 before the
 * first pass). */
int sc_ab2v_state(sc_handle* h, int* pass, double* dto);
/* The solvers' step rule, spectral_dns.f90:212-217: dt = min(betadx/umax,
 * 3 dto), cut to land on the output time twrite (halved when the remainder
 * would be under 0.2 dt).  Before the first pass the reference's dto is the
 * run's end time timemax (:111).  umax is theirs too: 3.5 sqrt(2E) every
 * ieout steps (:141; E from sc_diagnostics).  No GPU needed. */
int sc_ab2v_dt(double betadx, double umax, double dto, double time, double twrite, double* dt);

/* npasses passes of the rotating solver's loop, spectral_rot_dns_ft.f90:
 * 146-272 (replaces that program's time loop).  The state is the pair of
 * helical amplitudes a+ = v . conj(h), a- = v . h (heliwave.f90:57-96), each
 * advanced with exp(-nu k^2 dt +- 2 i dt kz om / |k|) (:101-111): pass 0 is
 * an Euler half step, pass 1 a midpoint restart from the initial field, then
 * AB2; after every pass the handle's state is v = a+ h + a- conj(h),
 * truncated at k >= kcut.  Right-hand side (:189-211): Lamb vector,
 * force_rot on the band fk1^2 <= k^2 < fk2^2 when the handle is forced
 * (eps from sc_params), symmetrize, projection.  om is the rotation rate.
 * The amplitudes (five extra fields with the previous right-hand side) are
 * allocated on the first call; sc_set_state and sc_init_field restart the
 * sequence at pass 0.  Handles with sgs != SC_SGS_NONE are rejected. */
int sc_rot_steps(sc_handle* h, int npasses, double om, double fk1, double fk2);

/* The passive scalar phi of the rotating scalar solver (reference layout,
 * host or device pointer).  Setting it restarts the rotating passes at 0;
 * before the first set it is zero. */
int sc_set_scalar(sc_handle* h, const void* phi);
int sc_get_scalar(sc_handle* h, void* phi);
/* npasses passes of the rotating solver with a passive scalar,
 * spectral_rot_dns_scalar_ft.f90:203-291 (that program does not compile as
 * written: its kx, ky, kz are declared rank 3 at :20 and allocated rank 1 at
 * :84; this is its evident intent with 1D wavenumbers).  Per pass: Lamb
 * vector and wphi = convecphi_dns; force_rot called with fk1, fk2 as its
 * squared bounds (band fk1 <= k^2 < fk2), as :213 does; when scalarforced,
 * forcephi_rot on fk1^2 <= k^2 < fk2^2 with epsphi; dealiasing of w and wphi;
 * projection; the helical AB2 of sc_rot_steps for v (not truncated after)
 * and the same schedule for phi with exp(-nu k^2 dt / pr).  Handles with
 * sgs != SC_SGS_NONE are rejected. */
int sc_rot_scalar_steps(sc_handle* h, int npasses, double om, double fk1, double fk2, double pr, int scalarforced,
                        double epsphi);

/* Discrete adjoint of nsteps IF-RK4 steps (DNS right-hand side) for
 * J = sum over shells kmin..kmax (floor(|k| + 1/2)) of k^2 q(k) at the final
 * time (q = 1/2-weighted |v|^2, the shell enstrophy).  Writes J and
 * dJ/dv_0 (host arrays, reference layout): g = dJ/dRe v + i dJ/dIm v for every
 * stored entry, so dJ = sum Re(conj(g) dv).  The state is checkpointed every
 * `checkpoint_every` steps and each segment is recomputed once, keeping its
 * stage inputs, before the backward sweep (segments within the memory budget
 * of sc_set_adjoint_budget keep them from the forward sweep instead).  The
 * handle's state is left at v_0.
 * No counterpart in the reference (its solvers have no adjoint). */
int sc_adjoint_rk4(sc_handle* h, int nsteps, int checkpoint_every, int kmin, int kmax, void* gx,
                   void* gy, void* gz, double* J);

/* Memory for the adjoint's stage-input store, in bytes (default -1: 90% of
 * the device memory free at the call).  The adjoint checkpoints the state
 * every `checkpoint_every` steps and recomputes a segment's stage inputs
 * before its backward sweep, except for the trailing segments whose stage
 * inputs (12 fields per step) fit this budget: the forward sweep keeps those.
 * 0 selects pure checkpointing.  sc_adjoint_kept_segments reports how many
 * segments the last adjoint call kept.  No reference counterpart. */
int sc_set_adjoint_budget(sc_handle* h, double bytes);
int sc_adjoint_kept_segments(sc_handle* h, int* kept);

/* Vector-Jacobian product of nsteps IF-RK4 steps: given lam_T (host arrays,
 * reference layout, same convention as the gradient above) returns
 * g = (dv_T/dv_0)^T lam_T for the handle's current state v_0, which is left
 * in place.  Same checkpointing as sc_adjoint_rk4.  No reference counterpart. */
int sc_adjoint_rk4_vjp(sc_handle* h, int nsteps, int checkpoint_every, const void* lx, const void* ly,
                       const void* lz, void* gx, void* gy, void* gz);

/* Fortran unformatted field files, as the reference's output3d / input3d
 * write and read them (output.f90:103-132, input.f90:106-136): the state goes
 * to <dir>/ux<idump>.dat, uy<idump>.dat, uz<idump>.dat ("./out" in the
 * reference), one sequential unformatted record each holding the
 * complex(sp) (nx/2+1, ny, nz) array in Fortran order.  file_precision
 * (SC_FP32 / SC_FP64) is the sp of the reference build that writes or reads
 * the files; values convert to and from the handle's precision.  sc_input3d
 * loads the state as sc_set_state does. */
int sc_output3d(sc_handle* h, const char* dir, int idump, int file_precision);
int sc_input3d(sc_handle* h, const char* dir, int idump, int file_precision);
/* The passive scalar as outputphi / inputphi write and read it
 * (outputphi.f90:1-20, inputphi.f90:1-22): <dir>/phi<idump>.dat, one record of
 * complex(sp) (nx/2+1, ny, nz); sc_inputphi loads it as sc_set_scalar does. */
int sc_outputphi(sc_handle* h, const char* dir, int idump, int file_precision);
int sc_inputphi(sc_handle* h, const char* dir, int idump, int file_precision);

/* One record of a gfortran sequential unformatted file, host memory only: a
 * 4-byte little-endian length marker, the bytes, the marker again; records
 * longer than max_subrecord bytes (0 = gfortran's 2147483639) are split into
 * subrecords, a leading marker negative when more follow and a trailing
 * marker negative when one precedes.  The reader follows the markers and
 * requires exactly nbytes of data. */
int sc_fortran_record_write(const char* path, const void* data, long long nbytes, long long max_subrecord);
int sc_fortran_record_read(const char* path, void* data, long long nbytes);

/* FP64 diagnostics of the current state; eks (may be NULL) receives the
 * shell spectrum E(k), k = 1..nx/2 (specdns-forced-omp-ft.f90:159-176). */
int sc_diagnostics(sc_handle* h, sc_diag* d, double* eks);

/* Per-kernel timing with CUDA events on the launching stream.
 * sc_profile_enable(h, 1) starts recording; sc_profile_read returns, for
 * kernel family `name` ("zinv","ypass_inv","xpass","ypass_fwd","zfwd",
 * "fixup", ...), the launch count and summed milliseconds since enabling. */
int sc_profile_enable(sc_handle* h, int on);
int sc_profile_read(sc_handle* h, const char* name, long long* launches, double* ms);

/* Algorithmic bytes (field-pass model) of one RK4 step for this handle. */
int sc_step_bytes(sc_handle* h, double* bytes_per_step);

/* No reference counterpart: a measurement helper.  Runs a bounded FP64 FMA
 * throughput kernel (eight independent fma chains per thread, four blocks of
 * 256 threads per SM) on the current device and returns the best rate of
 * three timed launches in TFLOP/s: the compute ceiling of the plain-FP64
 * step's roofline. */
int sc_fp64_peak_probe(double* tflops);

const char* sc_last_error(void);

/* ---------------------------------------------------------------------
 * Batched 2D vorticity ensembles.  Independent periodic 2D runs of mixed
 * size N (powers of two, 64..1024) advance together: vorticity w^ (N, N/2+1
 * complex, kx fastest), u^ = i ky w^/k^2, v^ = -i kx w^/k^2, nonlinear term
 * -(i kx (u w)^ + i ky (v w)^) with symmetrize2d (symmetrize.f90:8-30) and
 * the 2/3 mask, linear damping alpha and hyperviscosity nu8 (del^8) through
 * the integrating factor exp(-(alpha + nu8 k^8) dt/2) in the IF-RK4.  The
 * physics restates the reference's 2D solvers (spectral_dns_2d.f90:94,160-188,
 * turb_2d.f90:288-403); the reference has no ensemble driver.
 * ------------------------------------------------------------------- */
typedef struct sc_ensemble sc_ensemble;
int sc_ens_create(int precision, int nmembers, const int* n, const double* dt, const double* nu8,
                  double alpha, sc_ensemble** out);
int sc_ens_destroy(sc_ensemble* e);
int sc_ens_set_stream(sc_ensemble* e, void* stream);
/* member m's vorticity, host array (N, N/2+1) complex */
int sc_ens_set_member(sc_ensemble* e, int m, const void* w);
int sc_ens_get_member(sc_ensemble* e, int m, void* w);
/* seeded random vorticity with E(k) ~ k exp(-(k/kpeak)^2), energy `energy`
 * (ran1 draws in the order of initialize.f90:485-492, then symmetrize2d and
 * the 2/3 mask); seeds[m] per member (only seeds <= 0 select distinct ran1
 * streams, initialize.f90:530) */
int sc_ens_init(sc_ensemble* e, const int* seeds, double kpeak, double energy);
/* nsteps IF-RK4 steps of every member.  mode 0: one cooperative launch per
 * stage for all members, a whole step replayed as a CUDA graph; mode 1: the
 * same launches without the graph; mode 2: the members one at a time. */
int sc_ens_rk4_steps(sc_ensemble* e, int nsteps, int mode);
/* 1 if mode 0 is running from a captured graph */
int sc_ens_uses_graph(sc_ensemble* e);

/* Launch-shape autotuner.  The stage kernel is compiled in several shapes
 * (threads per CTA, CTAs per SM, points per y tile, largest FFT radix);
 * sc_ens_tune times each on this ensemble (`trial_steps` steps each, the
 * member states saved and restored) and keeps the fastest.  The first
 * sc_ens_rk4_steps call tunes with 3 trial steps unless a variant was set
 * (sc_ens_set_variant, or SPECNS_ENS_VARIANT) or SPECNS_ENS_TUNE=0.
 * Variants round differently (FP32 results agree to ~1e-6); pin one for
 * bit-reproducible runs.  sc_ens_variant reports the current variant, the
 * number of variants, the last tuning's ms per step per variant
 * (tune_ms[count], -1 = not timed) and the shape {threads, CTAs per SM,
 * tile points, radix, phases out of line} (shape[5]); any pointer may be
 * NULL.
 * No reference counterpart. */
int sc_ens_tune(sc_ensemble* e, int trial_steps, int* chosen);
int sc_ens_set_variant(sc_ensemble* e, int variant);
int sc_ens_variant(sc_ensemble* e, int* variant, int* count, double* tune_ms, int* shape);

/* No counterpart in the reference.  FP64 diagnostics of a caller-owned
 * spectral velocity field that allocate no device memory, for callers that
 * cannot call cudaMalloc: a solver that reserves its whole device-memory
 * budget at start-up and must not allocate inside its step loop, or one that
 * cannot afford the device-wide synchronisation cudaMalloc/cudaFree may
 * imply.  vx, vy, vz: device arrays in the reference layout (pitch nx/2+1),
 * complex(4) for SC_FP32, complex(8) for SC_FP64.  out: device array of
 * 5 + nx/2 doubles receiving [energy, sum k^2 q (enstrophy; dissipation =
 * 2 nu times it), max |k.v|, non-finite count, 0, E(1..nx/2)].  Enqueued on
 * `stream` (cudaStream_t as void*, NULL = default stream), asynchronous.
 * Block partial sums live in one static device array of 4.04 MiB per GPU
 * (held until exit), sized for nx, ny, nz <= 1024; larger grids are
 * rejected.  All calls share that array: calls that overlap on the GPU race.
 * The first call on a device looks up the array's address and keeps it for
 * the life of the process; make it before any stream capture.  The kept
 * address belongs to the device's primary context: after cudaDeviceReset
 * (or any other teardown of that context) it is stale, and this entry point
 * must not be called on that device again. */
int sc_diagnostics_noalloc(int precision, const void* vx, const void* vy, const void* vz, int nx,
                           int ny, int nz, double* out, void* stream);

/* ---------------------------------------------------------------------
 * Reference-signature operators (one call = one reference subroutine).
 * Arrays are host memory in the reference layout; integer sizes are passed
 * by value.  `precision` selects complex(4) or complex(8) element data.
 * ------------------------------------------------------------------- */

/* convec_dns(vx,vy,vz,wx,wy,wz,lx1,ly,lz,nx,ny,nz), convec_dns.f90:1:
 * w <- spectral Lamb vector u x w (inputs v^, w^ = vorticity). */
int sc_convec_dns(int precision, const void* vx, const void* vy, const void* vz, void* wx,
                  void* wy, void* wz, int lx1, int ly, int lz, int nx, int ny, int nz);

/* projection(vx,vy,vz,kx,ky,kz,lx1,ly,lz), projection.f90:2 (kx, ky, kz are
 * implied by the FFTW ordering and not passed). */
int sc_projection(int precision, void* vx, void* vy, void* vz, int lx1, int ly, int lz);

/* force(wx,wy,wz,vx,vy,vz,k2,lx1,ly,lz,fkmax,eps), force.f90:3 (k2 implied). */
int sc_force(int precision, void* wx, void* wy, void* wz, const void* vx, const void* vy,
             const void* vz, int lx1, int ly, int lz, double fkmax, double eps);

/* force_rot(wx,wy,wz,vx,vy,vz,k2,lx1,ly,lz,fk12,fk22,eps), force_rot.f90:3:
 * w += eps/(2 K + tiny) v on the shell band fk12 <= k^2 < fk22 (squared
 * bounds, as the reference passes them), K the band energy (FP64). */
int sc_force_rot(int precision, void* wx, void* wy, void* wz, const void* vx, const void* vy,
                 const void* vz, int lx1, int ly, int lz, double fk12, double fk22, double eps);
/* forcephi(phi,wphi,k2,lx1,ly,lz,fkmax,epsphi), forcephi.f90:1: the passive
 * scalar's forcing wphi += epsphi/(2 K) phi on k^2 < fkmax^2, K the
 * 1/2-weighted variance of phi there (FP64 sum); wphi in place. */
int sc_forcephi(int precision, const void* phi, void* wphi, int lx1, int ly, int lz, double fkmax, double epsphi);
/* forcephi_rot(phi,wphi,k2,lx1,ly,lz,fk1,fk2,epsphi), forcephi_rot.f90:1: the
 * same on the band fk1^2 <= k^2 < fk2^2. */
int sc_forcephi_rot(int precision, const void* phi, void* wphi, int lx1, int ly, int lz, double fk1, double fk2,
                    double epsphi);

/* convecphi_dns(vx,vy,vz,phi,wphi,kx,ky,kz,lx1,ly,lz,nx,ny,nz),
 * convecphi_dns.f90:1: wphi <- i k . (u phi)^ / N^3, the spectral flux
 * divergence of a passive scalar phi (kx, ky, kz implied). */
int sc_convecphi_dns(int precision, const void* vx, const void* vy, const void* vz, const void* phi,
                     void* wphi, int lx1, int ly, int lz, int nx, int ny, int nz);

/* skewness(ux,kx,s,nx,ny,nz), skewness.f90:1: S = <d^3> / <d^2>^(3/2) of
 * d = du_x/dx over the physical grid (moments summed in FP64). */
int sc_skewness(int precision, const void* ux, int nx, int ny, int nz, double* s);

/* enstrophy(ux,uy,uz,kx,ky,kz,enstr,lx1,ly,lz,lx,nx,ny,nz), enstrophy.f90:1:
 * enstr = 1/2 |w|^2, w = curl u, at every physical point; enstr is real(dp)
 * (nx, ny, nz) in Fortran order. */
int sc_enstrophy(int precision, const void* ux, const void* uy, const void* uz, double* enstr, int lx1,
                 int ly, int lz, int nx, int ny, int nz);

/* symmetrize(c,lx1,ly,lz), symmetrize.f90:32 (3D). */
int sc_symmetrize(int precision, void* c, int lx1, int ly, int lz);

/* dealiasing(c,k2,lx1,ly,lz), dealiasing.f90:2. */
/* hermitianize(c,lx1,ly,lz), hermitianize.f90:1: the kx = 0 plane's conjugate
 * symmetry c(1,iy,iz) = conj(c(1,-iy,-iz)) for iz > lz/2 and on the line
 * kz = 0, iy > ly/2, without symmetrize's zeroing; c in place. */
int sc_hermitianize(int precision, void* c, int lx1, int ly, int lz);
int sc_dealiasing(int precision, void* c, int lx1, int ly, int lz);

/* smag(vx,vy,vz,t11,t12,t13,t22,t23,t33,kx,ky,kz,lx1,ly,lz,nx,ny,nz,delta),
 * smag.f90:1, with c1 an argument (the reference fixes 0.026). */
int sc_smag(int precision, const void* vx, const void* vy, const void* vz, void* t11, void* t12,
            void* t13, void* t22, void* t23, void* t33, int lx1, int ly, int lz, int nx, int ny,
            int nz, double delta, double c1);

/* dynsmag(ux,uy,uz,t11..t33,kx,ky,kz,g_test,lx1,ly,lz,nx,ny,nz,lx,delta,
 * delta_test,mm,lm,cs2,update), dynsmag.f90:1.  g_test is the sharp filter
 * k2 <= k_test^2 (spectral_les.f90:105-109), passed as k_test.  cs2 is read
 * when update == 0 and written otherwise, with mm and lm. */
int sc_dynsmag(int precision, const void* ux, const void* uy, const void* uz, void* t11,
               void* t12, void* t13, void* t22, void* t23, void* t33, int lx1, int ly, int lz,
               int nx, int ny, int nz, double k_test, double delta, double delta_test,
               double* mm, double* lm, double* cs2, int update);

#ifdef __cplusplus
}
#endif
#endif /* SPECNS_H */
