! specns.f90 -- ISO_C_BINDING interfaces of libspecns.so (include/specns.h)
! for Fortran solver programs: the handle API, the steppers, the
! reference-signature operators, the 2D ensembles.  Arrays are passed as
! assumed-type arguments (TYPE(*)), so one module serves complex(4) and
! complex(8) fields: the precision is the handle's (sc_params%precision) or
! the operator's first argument.  Strings are C strings: pass
! trim(name)//c_null_char.  Every function returns SC_OK or an SC_ERR_* code;
! sc_last_error returns the message as a C pointer (c_f_pointer to read it).
module specns
  use, intrinsic :: iso_c_binding
  implicit none

  integer(c_int), parameter :: SC_OK = 0
  integer(c_int), parameter :: SC_ERR_INVALID = 1
  integer(c_int), parameter :: SC_ERR_CUDA = 2
  integer(c_int), parameter :: SC_ERR_NONFINITE = 3
  integer(c_int), parameter :: SC_ERR_TIMEOUT = 4
  integer(c_int), parameter :: SC_ERR_NOMEM = 5
  integer(c_int), parameter :: SC_ERR_IO = 6
  integer(c_int), parameter :: SC_FP32 = 0
  integer(c_int), parameter :: SC_FP64 = 1
  integer(c_int), parameter :: SC_SGS_NONE = 0
  integer(c_int), parameter :: SC_SGS_SMAG = 1
  integer(c_int), parameter :: SC_SGS_DYNSMAG = 2
  integer(c_int), parameter :: SC_MASK_AFTER_STEP = 0
  integer(c_int), parameter :: SC_MASK_RHS_AND_STEP = 1

  type, bind(C) :: sc_params
    integer(c_int) :: nx, ny, nz, precision
    real(c_double) :: nu, dt
    integer(c_int) :: forced
    real(c_double) :: eps, fkmax, kcut
    integer(c_int) :: sgs
    real(c_double) :: c1, delta, delta_ratio
    integer(c_int) :: dyn_every, mask_mode
  end type sc_params

  type, bind(C) :: sc_diag
    real(c_double) :: energy, enstrophy, dissipation, max_div, max_u, nonfinite, cs2, mm, lm
  end type sc_diag

  interface
    integer(c_int) function sc_default_params(p, n, precision) bind(C, name="sc_default_params")
      import
      type(sc_params) :: p
      integer(c_int), value :: n
      integer(c_int), value :: precision
    end function sc_default_params
    integer(c_int) function sc_create(p, out) bind(C, name="sc_create")
      import
      type(sc_params), intent(in) :: p
      type(c_ptr), intent(out) :: out
    end function sc_create
    integer(c_int) function sc_destroy(h) bind(C, name="sc_destroy")
      import
      type(c_ptr), value :: h
    end function sc_destroy
    integer(c_int) function sc_set_device(device) bind(C, name="sc_set_device")
      import
      integer(c_int), value :: device
    end function sc_set_device
    integer(c_int) function sc_set_stream(h, stream) bind(C, name="sc_set_stream")
      import
      type(c_ptr), value :: h
      type(c_ptr), value :: stream
    end function sc_set_stream
    integer(c_int) function sc_set_dt(h, dt) bind(C, name="sc_set_dt")
      import
      type(c_ptr), value :: h
      real(c_double), value :: dt
    end function sc_set_dt
    integer(c_int) function sc_get_params(h, out) bind(C, name="sc_get_params")
      import
      type(c_ptr), value :: h
      type(sc_params) :: out
    end function sc_get_params
    integer(c_int) function sc_set_state(h, vx, vy, vz) bind(C, name="sc_set_state")
      import
      type(c_ptr), value :: h
      type(*), dimension(*), intent(in) :: vx
      type(*), dimension(*), intent(in) :: vy
      type(*), dimension(*), intent(in) :: vz
    end function sc_set_state
    integer(c_int) function sc_get_state(h, vx, vy, vz) bind(C, name="sc_get_state")
      import
      type(c_ptr), value :: h
      type(*), dimension(*) :: vx
      type(*), dimension(*) :: vy
      type(*), dimension(*) :: vz
    end function sc_get_state
    integer(c_int) function sc_set_state_device(h, vx, vy, vz) bind(C, name="sc_set_state_device")
      import
      type(c_ptr), value :: h
      type(*), dimension(*), intent(in) :: vx
      type(*), dimension(*), intent(in) :: vy
      type(*), dimension(*), intent(in) :: vz
    end function sc_set_state_device
    integer(c_int) function sc_get_state_device(h, vx, vy, vz) bind(C, name="sc_get_state_device")
      import
      type(c_ptr), value :: h
      type(*), dimension(*) :: vx
      type(*), dimension(*) :: vy
      type(*), dimension(*) :: vz
    end function sc_get_state_device
    integer(c_int) function sc_init_field(h, seed, kind, akp, u0, kmin, kmax) bind(C, name="sc_init_field")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: seed
      integer(c_int), value :: kind
      real(c_double), value :: akp
      real(c_double), value :: u0
      real(c_double), value :: kmin
      real(c_double), value :: kmax
    end function sc_init_field
    integer(c_int) function sc_rhs(h, wx, wy, wz) bind(C, name="sc_rhs")
      import
      type(c_ptr), value :: h
      type(*), dimension(*) :: wx
      type(*), dimension(*) :: wy
      type(*), dimension(*) :: wz
    end function sc_rhs
    integer(c_int) function sc_rk4_steps(h, nsteps) bind(C, name="sc_rk4_steps")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
    end function sc_rk4_steps
    integer(c_int) function sc_ab2_steps(h, npasses) bind(C, name="sc_ab2_steps")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: npasses
    end function sc_ab2_steps
    integer(c_int) function sc_ab2v_pass(h, dt) bind(C, name="sc_ab2v_pass")
      import
      type(c_ptr), value :: h
      real(c_double), value :: dt
    end function sc_ab2v_pass
    integer(c_int) function sc_ab2v_scalar_pass(h, dt, pr, scalarforced, meangrad, history_rhs) bind(C, &
        name="sc_ab2v_scalar_pass")
      import
      type(c_ptr), value :: h
      real(c_double), value :: dt
      real(c_double), value :: pr
      integer(c_int), value :: scalarforced
      real(c_double), value :: meangrad
      integer(c_int), value :: history_rhs
    end function sc_ab2v_scalar_pass
    integer(c_int) function sc_ab2v_state(h, pass, dto) bind(C, name="sc_ab2v_state")
      import
      type(c_ptr), value :: h
      integer(c_int), intent(out) :: pass
      real(c_double), intent(out) :: dto
    end function sc_ab2v_state
    integer(c_int) function sc_ab2v_dt(betadx, umax, dto, time, twrite, dt) bind(C, name="sc_ab2v_dt")
      import
      real(c_double), value :: betadx
      real(c_double), value :: umax
      real(c_double), value :: dto
      real(c_double), value :: time
      real(c_double), value :: twrite
      real(c_double), intent(out) :: dt
    end function sc_ab2v_dt
    integer(c_int) function sc_rot_steps(h, npasses, om, fk1, fk2) bind(C, name="sc_rot_steps")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: npasses
      real(c_double), value :: om
      real(c_double), value :: fk1
      real(c_double), value :: fk2
    end function sc_rot_steps
    integer(c_int) function sc_set_scalar(h, phi) bind(C, name="sc_set_scalar")
      import
      type(c_ptr), value :: h
      type(*), dimension(*), intent(in) :: phi
    end function sc_set_scalar
    integer(c_int) function sc_get_scalar(h, phi) bind(C, name="sc_get_scalar")
      import
      type(c_ptr), value :: h
      type(*), dimension(*) :: phi
    end function sc_get_scalar
    integer(c_int) function sc_rot_scalar_steps(h, npasses, om, fk1, fk2, pr, scalarforced, epsphi) bind(C, &
        name="sc_rot_scalar_steps")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: npasses
      real(c_double), value :: om
      real(c_double), value :: fk1
      real(c_double), value :: fk2
      real(c_double), value :: pr
      integer(c_int), value :: scalarforced
      real(c_double), value :: epsphi
    end function sc_rot_scalar_steps
    integer(c_int) function sc_adjoint_rk4(h, nsteps, checkpoint_every, kmin, kmax, gx, gy, gz, jval) bind(C, &
        name="sc_adjoint_rk4")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
      integer(c_int), value :: checkpoint_every
      integer(c_int), value :: kmin
      integer(c_int), value :: kmax
      type(*), dimension(*) :: gx
      type(*), dimension(*) :: gy
      type(*), dimension(*) :: gz
      real(c_double), intent(out) :: jval
    end function sc_adjoint_rk4
    integer(c_int) function sc_set_adjoint_budget(h, bytes) bind(C, name="sc_set_adjoint_budget")
      import
      type(c_ptr), value :: h
      real(c_double), value :: bytes
    end function sc_set_adjoint_budget
    integer(c_int) function sc_adjoint_kept_segments(h, kept) bind(C, name="sc_adjoint_kept_segments")
      import
      type(c_ptr), value :: h
      integer(c_int), intent(out) :: kept
    end function sc_adjoint_kept_segments
    integer(c_int) function sc_adjoint_rk4_vjp(h, nsteps, checkpoint_every, lamx, lamy, lamz, gx, gy, &
        gz) bind(C, name="sc_adjoint_rk4_vjp")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: nsteps
      integer(c_int), value :: checkpoint_every
      type(*), dimension(*), intent(in) :: lamx
      type(*), dimension(*), intent(in) :: lamy
      type(*), dimension(*), intent(in) :: lamz
      type(*), dimension(*) :: gx
      type(*), dimension(*) :: gy
      type(*), dimension(*) :: gz
    end function sc_adjoint_rk4_vjp
    integer(c_int) function sc_output3d(h, dir, idump, file_precision) bind(C, name="sc_output3d")
      import
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*), intent(in) :: dir
      integer(c_int), value :: idump
      integer(c_int), value :: file_precision
    end function sc_output3d
    integer(c_int) function sc_input3d(h, dir, idump, file_precision) bind(C, name="sc_input3d")
      import
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*), intent(in) :: dir
      integer(c_int), value :: idump
      integer(c_int), value :: file_precision
    end function sc_input3d
    integer(c_int) function sc_outputphi(h, dir, idump, file_precision) bind(C, name="sc_outputphi")
      import
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*), intent(in) :: dir
      integer(c_int), value :: idump
      integer(c_int), value :: file_precision
    end function sc_outputphi
    integer(c_int) function sc_inputphi(h, dir, idump, file_precision) bind(C, name="sc_inputphi")
      import
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*), intent(in) :: dir
      integer(c_int), value :: idump
      integer(c_int), value :: file_precision
    end function sc_inputphi
    integer(c_int) function sc_fortran_record_write(path, data, nbytes, max_subrecord) bind(C, &
        name="sc_fortran_record_write")
      import
      character(kind=c_char), dimension(*), intent(in) :: path
      type(*), dimension(*), intent(in) :: data
      integer(c_long_long), value :: nbytes
      integer(c_long_long), value :: max_subrecord
    end function sc_fortran_record_write
    integer(c_int) function sc_fortran_record_read(path, data, nbytes) bind(C, name="sc_fortran_record_read")
      import
      character(kind=c_char), dimension(*), intent(in) :: path
      type(*), dimension(*) :: data
      integer(c_long_long), value :: nbytes
    end function sc_fortran_record_read
    integer(c_int) function sc_diagnostics(h, d, eks) bind(C, name="sc_diagnostics")
      import
      type(c_ptr), value :: h
      type(sc_diag), intent(out) :: d
      real(c_double), dimension(*) :: eks
    end function sc_diagnostics
    integer(c_int) function sc_profile_enable(h, on) bind(C, name="sc_profile_enable")
      import
      type(c_ptr), value :: h
      integer(c_int), value :: on
    end function sc_profile_enable
    integer(c_int) function sc_profile_read(h, name, launches, ms) bind(C, name="sc_profile_read")
      import
      type(c_ptr), value :: h
      character(kind=c_char), dimension(*), intent(in) :: name
      integer(c_long_long), intent(out) :: launches
      real(c_double), intent(out) :: ms
    end function sc_profile_read
    integer(c_int) function sc_step_bytes(h, bytes_per_step) bind(C, name="sc_step_bytes")
      import
      type(c_ptr), value :: h
      real(c_double), intent(out) :: bytes_per_step
    end function sc_step_bytes
    integer(c_int) function sc_fp64_peak_probe(tflops) bind(C, name="sc_fp64_peak_probe")
      import
      real(c_double), intent(out) :: tflops
    end function sc_fp64_peak_probe
    type(c_ptr) function sc_last_error() bind(C, name="sc_last_error")
      import
    end function sc_last_error
    integer(c_int) function sc_ens_create(precision, nmembers, n, dt, nu8, alpha, out) bind(C, name="sc_ens_create")
      import
      integer(c_int), value :: precision
      integer(c_int), value :: nmembers
      integer(c_int), dimension(*), intent(in) :: n
      real(c_double), dimension(*), intent(in) :: dt
      real(c_double), dimension(*), intent(in) :: nu8
      real(c_double), value :: alpha
      type(c_ptr), intent(out) :: out
    end function sc_ens_create
    integer(c_int) function sc_ens_destroy(e) bind(C, name="sc_ens_destroy")
      import
      type(c_ptr), value :: e
    end function sc_ens_destroy
    integer(c_int) function sc_ens_set_stream(e, stream) bind(C, name="sc_ens_set_stream")
      import
      type(c_ptr), value :: e
      type(c_ptr), value :: stream
    end function sc_ens_set_stream
    integer(c_int) function sc_ens_set_member(e, m, w) bind(C, name="sc_ens_set_member")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: m
      type(*), dimension(*), intent(in) :: w
    end function sc_ens_set_member
    integer(c_int) function sc_ens_get_member(e, m, w) bind(C, name="sc_ens_get_member")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: m
      type(*), dimension(*) :: w
    end function sc_ens_get_member
    integer(c_int) function sc_ens_init(e, seeds, kpeak, energy) bind(C, name="sc_ens_init")
      import
      type(c_ptr), value :: e
      integer(c_int), dimension(*), intent(in) :: seeds
      real(c_double), value :: kpeak
      real(c_double), value :: energy
    end function sc_ens_init
    integer(c_int) function sc_ens_rk4_steps(e, nsteps, mode) bind(C, name="sc_ens_rk4_steps")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: nsteps
      integer(c_int), value :: mode
    end function sc_ens_rk4_steps
    integer(c_int) function sc_ens_uses_graph(e) bind(C, name="sc_ens_uses_graph")
      import
      type(c_ptr), value :: e
    end function sc_ens_uses_graph
    integer(c_int) function sc_ens_tune(e, trial_steps, chosen) bind(C, name="sc_ens_tune")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: trial_steps
      integer(c_int), intent(out) :: chosen
    end function sc_ens_tune
    integer(c_int) function sc_ens_set_variant(e, variant) bind(C, name="sc_ens_set_variant")
      import
      type(c_ptr), value :: e
      integer(c_int), value :: variant
    end function sc_ens_set_variant
    integer(c_int) function sc_ens_variant(e, variant, count, tune_ms, shape) bind(C, name="sc_ens_variant")
      import
      type(c_ptr), value :: e
      integer(c_int), intent(out) :: variant
      integer(c_int), intent(out) :: count
      real(c_double), dimension(*) :: tune_ms
      integer(c_int), dimension(*) :: shape
    end function sc_ens_variant
    integer(c_int) function sc_diagnostics_noalloc(precision, vx, vy, vz, nx, ny, nz, out, stream) bind(C, &
        name="sc_diagnostics_noalloc")
      import
      integer(c_int), value :: precision
      type(*), dimension(*), intent(in) :: vx
      type(*), dimension(*), intent(in) :: vy
      type(*), dimension(*), intent(in) :: vz
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      real(c_double), dimension(*) :: out
      type(c_ptr), value :: stream
    end function sc_diagnostics_noalloc
    integer(c_int) function sc_convec_dns(precision, vx, vy, vz, wx, wy, wz, lx1, ly, lz, nx, ny, nz) bind(C, &
        name="sc_convec_dns")
      import
      integer(c_int), value :: precision
      type(*), dimension(*), intent(in) :: vx
      type(*), dimension(*), intent(in) :: vy
      type(*), dimension(*), intent(in) :: vz
      type(*), dimension(*) :: wx
      type(*), dimension(*) :: wy
      type(*), dimension(*) :: wz
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
    end function sc_convec_dns
    integer(c_int) function sc_projection(precision, vx, vy, vz, lx1, ly, lz) bind(C, name="sc_projection")
      import
      integer(c_int), value :: precision
      type(*), dimension(*) :: vx
      type(*), dimension(*) :: vy
      type(*), dimension(*) :: vz
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
    end function sc_projection
    integer(c_int) function sc_force(precision, wx, wy, wz, vx, vy, vz, lx1, ly, lz, fkmax, eps) bind(C, &
        name="sc_force")
      import
      integer(c_int), value :: precision
      type(*), dimension(*) :: wx
      type(*), dimension(*) :: wy
      type(*), dimension(*) :: wz
      type(*), dimension(*), intent(in) :: vx
      type(*), dimension(*), intent(in) :: vy
      type(*), dimension(*), intent(in) :: vz
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
      real(c_double), value :: fkmax
      real(c_double), value :: eps
    end function sc_force
    integer(c_int) function sc_force_rot(precision, wx, wy, wz, vx, vy, vz, lx1, ly, lz, fk12, fk22, &
        eps) bind(C, name="sc_force_rot")
      import
      integer(c_int), value :: precision
      type(*), dimension(*) :: wx
      type(*), dimension(*) :: wy
      type(*), dimension(*) :: wz
      type(*), dimension(*), intent(in) :: vx
      type(*), dimension(*), intent(in) :: vy
      type(*), dimension(*), intent(in) :: vz
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
      real(c_double), value :: fk12
      real(c_double), value :: fk22
      real(c_double), value :: eps
    end function sc_force_rot
    integer(c_int) function sc_forcephi(precision, phi, wphi, lx1, ly, lz, fkmax, epsphi) bind(C, name="sc_forcephi")
      import
      integer(c_int), value :: precision
      type(*), dimension(*), intent(in) :: phi
      type(*), dimension(*) :: wphi
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
      real(c_double), value :: fkmax
      real(c_double), value :: epsphi
    end function sc_forcephi
    integer(c_int) function sc_forcephi_rot(precision, phi, wphi, lx1, ly, lz, fk1, fk2, epsphi) bind(C, &
        name="sc_forcephi_rot")
      import
      integer(c_int), value :: precision
      type(*), dimension(*), intent(in) :: phi
      type(*), dimension(*) :: wphi
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
      real(c_double), value :: fk1
      real(c_double), value :: fk2
      real(c_double), value :: epsphi
    end function sc_forcephi_rot
    integer(c_int) function sc_convecphi_dns(precision, vx, vy, vz, phi, wphi, lx1, ly, lz, nx, ny, &
        nz) bind(C, name="sc_convecphi_dns")
      import
      integer(c_int), value :: precision
      type(*), dimension(*), intent(in) :: vx
      type(*), dimension(*), intent(in) :: vy
      type(*), dimension(*), intent(in) :: vz
      type(*), dimension(*), intent(in) :: phi
      type(*), dimension(*) :: wphi
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
    end function sc_convecphi_dns
    integer(c_int) function sc_skewness(precision, ux, nx, ny, nz, s) bind(C, name="sc_skewness")
      import
      integer(c_int), value :: precision
      type(*), dimension(*), intent(in) :: ux
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      real(c_double), intent(out) :: s
    end function sc_skewness
    integer(c_int) function sc_enstrophy(precision, ux, uy, uz, enstr, lx1, ly, lz, nx, ny, nz) bind(C, &
        name="sc_enstrophy")
      import
      integer(c_int), value :: precision
      type(*), dimension(*), intent(in) :: ux
      type(*), dimension(*), intent(in) :: uy
      type(*), dimension(*), intent(in) :: uz
      real(c_double), dimension(*) :: enstr
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
    end function sc_enstrophy
    integer(c_int) function sc_symmetrize(precision, c, lx1, ly, lz) bind(C, name="sc_symmetrize")
      import
      integer(c_int), value :: precision
      type(*), dimension(*) :: c
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
    end function sc_symmetrize
    integer(c_int) function sc_hermitianize(precision, c, lx1, ly, lz) bind(C, name="sc_hermitianize")
      import
      integer(c_int), value :: precision
      type(*), dimension(*) :: c
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
    end function sc_hermitianize
    integer(c_int) function sc_dealiasing(precision, c, lx1, ly, lz) bind(C, name="sc_dealiasing")
      import
      integer(c_int), value :: precision
      type(*), dimension(*) :: c
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
    end function sc_dealiasing
    integer(c_int) function sc_smag(precision, vx, vy, vz, t11, t12, t13, t22, t23, t33, lx1, ly, lz, nx, ny, &
        nz, delta, c1) bind(C, name="sc_smag")
      import
      integer(c_int), value :: precision
      type(*), dimension(*), intent(in) :: vx
      type(*), dimension(*), intent(in) :: vy
      type(*), dimension(*), intent(in) :: vz
      type(*), dimension(*) :: t11
      type(*), dimension(*) :: t12
      type(*), dimension(*) :: t13
      type(*), dimension(*) :: t22
      type(*), dimension(*) :: t23
      type(*), dimension(*) :: t33
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      real(c_double), value :: delta
      real(c_double), value :: c1
    end function sc_smag
    integer(c_int) function sc_dynsmag(precision, ux, uy, uz, t11, t12, t13, t22, t23, t33, lx1, ly, lz, nx, &
        ny, nz, k_test, delta, delta_test, mm, lm, cs2, update) bind(C, name="sc_dynsmag")
      import
      integer(c_int), value :: precision
      type(*), dimension(*), intent(in) :: ux
      type(*), dimension(*), intent(in) :: uy
      type(*), dimension(*), intent(in) :: uz
      type(*), dimension(*) :: t11
      type(*), dimension(*) :: t12
      type(*), dimension(*) :: t13
      type(*), dimension(*) :: t22
      type(*), dimension(*) :: t23
      type(*), dimension(*) :: t33
      integer(c_int), value :: lx1
      integer(c_int), value :: ly
      integer(c_int), value :: lz
      integer(c_int), value :: nx
      integer(c_int), value :: ny
      integer(c_int), value :: nz
      real(c_double), value :: k_test
      real(c_double), value :: delta
      real(c_double), value :: delta_test
      real(c_double), intent(out) :: mm
      real(c_double), intent(out) :: lm
      real(c_double), intent(inout) :: cs2
      integer(c_int), value :: update
    end function sc_dynsmag
  end interface
end module specns
