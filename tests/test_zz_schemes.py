"""GPU parity of the rotating solver (spectral_rot_dns_ft.f90), its passive
scalar (spectral_rot_dns_scalar_ft.f90), the scalar forcing operators
(forcephi.f90, forcephi_rot.f90, also through their f77 shims) and the
variable-step IF-AB2 (spectral_dns.f90, spectral_les.f90) against the FP64
oracle.  Targets as for the other steppers: FP64 relative L2 <= 1e-12
(1e-11 with an SGS model), FP32 <= 1e-5 (2e-5 with an SGS model).

Collected after every other test file (file name), so that a run which stops
at its first failure has run the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import spectral_ref as R
from speccodelib_gb300 import _lib
from _util import complex_noise, fresh, hermitian_fields, rel_l2, solenoidal_init

pytestmark = pytest.mark.gpu

PRECS = [S.SC_FP64, S.SC_FP32]
TOL = {S.SC_FP64: 1e-12, S.SC_FP32: 1e-5}


def handle(n, prec, **kw):
    return S.SpectralNS(S.default_params(n, prec, **kw))


def oracle_grid(n, **kw):
    return R.Grid(R.Params(nx=n, **kw))


def cast(fields, prec):
    dt = np.complex128 if prec == S.SC_FP64 else np.complex64
    return [fresh(a, dt) for a in fields]


def ref_int(*xs):
    return [C.byref(C.c_int(x)) for x in xs]


@pytest.mark.parametrize("prec", PRECS)
def test_rotating_solver_matches_oracle(specns_lib, prec):
    """Five passes of the rotating solver's helical-wave IF-AB2
    (spectral_rot_dns_ft.f90:146-272) with band forcing 1 <= |k| < 2.5, and a
    restart through set_state, against the oracle."""
    n, om = 32, 5.0
    v = solenoidal_init(n)
    g = oracle_grid(n, nu=0.01, dt=2e-3, forced=True, eps=0.1)
    ref, _, _ = R.rot_run(v, g, 5, om, 1.0, 2.5)
    ref2, _, _ = R.rot_run(v, g, 2, om, 1.0, 2.5)
    with handle(n, prec, nu=0.01, dt=2e-3, forced=1, eps=0.1) as h:
        h.set_state(*v)
        h.rot_steps(5, om=om, fk1=1.0, fk2=2.5)
        out = h.get_state()
        h.set_state(*v)
        h.rot_steps(2, om=om, fk1=1.0, fk2=2.5)
        out2 = h.get_state()
    assert rel_l2(out, ref) < TOL[prec]
    assert rel_l2(out2, ref2) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("shape,band", [((32, 32, 32), (0.0, 2.5)), ((64, 32, 16), (1.0, 4.0)),
                                        ((128, 32, 32), (2.0, 5.0))])
def test_rotating_update_in_epilogue_and_separate(specns_lib, prec, shape, band, monkeypatch):
    """The rotating pass with force_rot's coefficient summed on the device
    and force_rot, symmetrize and projection in the z-forward epilogue
    (default), and with host-side band sums and a kernel for each of those
    operators (SPECNS_NO_FUSE_STEPPERS=1): both give the oracle's passes, on
    cubic and non-cubic grids, bands with and without the mean mode."""
    nx, ny, nz = shape
    fk1, fk2 = band
    v = hermitian_fields(shape, 71, kcut=2 * (nx // 2) / 3)
    kx, ky, kz, _ = R.wavenumber(nx, ny, nz)
    v = [R.symmetrize3d(a) for a in R.projection(*v, kx, ky, kz)]
    g = R.Grid(R.Params(nx=nx, ny=ny, nz=nz, nu=0.02, dt=2e-3, forced=True, eps=0.1))
    ref, _, _ = R.rot_run(v, g, 4, 4.0, fk1, fk2)
    outs = []
    for env in ("0", "1"):
        monkeypatch.setenv("SPECNS_NO_FUSE_STEPPERS", env)
        with S.SpectralNS(S.default_params(nx, prec, ny=ny, nz=nz, nu=0.02, dt=2e-3, forced=1, eps=0.1)) as h:
            h.set_state(*v)
            h.rot_steps(4, om=4.0, fk1=fk1, fk2=fk2)
            outs.append(h.get_state())
    for o in outs:
        assert rel_l2(o, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("shape", [(32, 32, 32), (64, 32, 16)])
def test_rotating_scalar_epilogue_and_separate(specns_lib, prec, shape, monkeypatch):
    """The rotating pass with a passive scalar: the velocity's right-hand
    side with force_rot (unsquared bounds), symmetrize, projection and the
    dealiasing mask in the z-forward epilogue (default), and with a kernel
    for each operator (SPECNS_NO_FUSE_STEPPERS=1): both give the oracle's
    velocity and scalar."""
    nx, ny, nz = shape
    pr = 0.7
    v = hermitian_fields(shape, 75, kcut=2 * (nx // 2) / 3)
    kx, ky, kz, k2 = R.wavenumber(nx, ny, nz)
    v = [R.symmetrize3d(a) for a in R.projection(*v, kx, ky, kz)]
    phi = R.dealiasing(hermitian_fields(shape, 76, ncomp=1)[0], k2)
    g = R.Grid(R.Params(nx=nx, ny=ny, nz=nz, nu=0.01, dt=2e-3, forced=True, eps=0.1))
    ref_v, ref_phi, _, _ = R.rot_scalar_run(v, phi, g, 4, 5.0, 1.0, 2.5, pr, True, 0.05)
    for env in ("0", "1"):
        monkeypatch.setenv("SPECNS_NO_FUSE_STEPPERS", env)
        with S.SpectralNS(S.default_params(nx, prec, ny=ny, nz=nz, nu=0.01, dt=2e-3, forced=1, eps=0.1)) as h:
            h.set_state(*v)
            h.set_scalar(phi)
            h.rot_scalar_steps(4, om=5.0, fk1=1.0, fk2=2.5, pr=pr, scalarforced=True, epsphi=0.05)
            assert rel_l2(h.get_state(), ref_v) < TOL[prec], env
            assert rel_l2(h.get_scalar(), ref_phi) < TOL[prec], env


@pytest.mark.parametrize("prec", PRECS)
def test_rotating_passes_replayed_from_a_graph(specns_lib, prec, monkeypatch):
    """From pass 2 on, sc_rot_steps replays one captured pass; the state is
    bit-identical to launching every kernel (SPECNS_NO_GRAPH=1), across calls,
    a change of om (a new capture) and a restart through set_state."""
    n = 32
    v = solenoidal_init(n)
    outs = []
    for env in ("0", "1"):
        monkeypatch.setenv("SPECNS_NO_GRAPH", env)
        with handle(n, prec, nu=0.01, dt=2e-3, forced=1, eps=0.1) as h:
            h.set_state(*v)
            h.rot_steps(5, om=5.0, fk1=1.0, fk2=2.5)
            h.rot_steps(3, om=5.0, fk1=1.0, fk2=2.5)
            h.rot_steps(2, om=2.0, fk1=1.0, fk2=2.5)
            a = h.get_state()
            h.set_state(*v)
            h.rot_steps(4, om=5.0, fk1=0.0, fk2=3.0)
            outs.append((a, h.get_state()))
    assert rel_l2(outs[0][0], outs[1][0]) == 0.0
    assert rel_l2(outs[0][1], outs[1][1]) == 0.0


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("shape", [(32, 32, 32), (64, 16, 32)])
def test_variable_step_update_in_epilogue_and_separate(specns_lib, prec, shape, monkeypatch):
    """The variable-step IF-AB2 with its update in the z-forward epilogue
    (default) and in its own kernel (SPECNS_NO_FUSE_STEPPERS=1): both give
    the oracle's passes over an uneven step sequence."""
    nx, ny, nz = shape
    v = hermitian_fields(shape, 73, kcut=2 * (nx // 2) / 3)
    kx, ky, kz, _ = R.wavenumber(nx, ny, nz)
    v = [R.symmetrize3d(a) for a in R.projection(*v, kx, ky, kz)]
    g = R.Grid(R.Params(nx=nx, ny=ny, nz=nz, nu=0.01, forced=True, eps=0.1, kcut=nx // 2))
    ref, _, _ = R.ab2v_run(v, g, STEPS_V)
    outs = []
    for env in ("0", "1"):
        monkeypatch.setenv("SPECNS_NO_FUSE_STEPPERS", env)
        with S.SpectralNS(S.default_params(nx, prec, ny=ny, nz=nz, nu=0.01, forced=1, eps=0.1,
                                           kcut=nx // 2)) as h:
            h.set_state(*v)
            for dt in STEPS_V:
                h.ab2v_pass(dt)
            outs.append(h.get_state())
    for o in outs:
        assert rel_l2(o, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_rotating_solver_beltrami_inertial_waves(specns_lib, prec):
    """An ABC (Beltrami, curl u = u) flow has a zero Lamb vector, so the
    rotating solver advances its helical amplitudes by the integrating factor
    alone: after p >= 2 passes a+ = a+(0) exp(-nu (p-1) dt + 2 i kz om
    (p-1) dt / |k|), and v = a+ h."""
    n, om, nu, dt, npass = 16, 3.0, 0.05, 1e-2, 7
    z, y, x = np.meshgrid(*[np.arange(n) * 2 * np.pi / n for _ in range(3)], indexing="ij")
    A, B, Cc = 1.0, 0.7, 0.4
    u = [A * np.sin(z) + Cc * np.cos(y), B * np.sin(x) + A * np.cos(z), Cc * np.sin(y) + B * np.cos(x)]
    v = [R.r2c(a) / n ** 3 for a in u]
    kx, ky, kz, k2 = R.wavenumber(n, n, n)
    h = R.heliwave(kx, ky, kz, k2)
    ap0 = sum(a * np.conj(b) for a, b in zip(v, h))
    ph = np.exp(-nu * (npass - 1) * dt + 2j * kz[:, None, None] * om * (npass - 1) * dt / np.sqrt(k2))
    exact = [ap0 * ph * b for b in h]
    with handle(n, prec, nu=nu, dt=dt, forced=0) as hd:
        hd.set_state(*v)
        hd.rot_steps(npass, om=om)
        out = hd.get_state()
    assert rel_l2(out, exact) < (1e-13 if prec == S.SC_FP64 else TOL[prec])


STEPS_V = [2e-3, 2.6e-3, 1.4e-3, 2.2e-3, 1.8e-3, 2.4e-3]


@pytest.mark.parametrize("prec", PRECS)
def test_variable_step_ab2_matches_oracle(specns_lib, prec):
    """Passes of spectral_dns.f90's variable-step IF-AB2 on an uneven step
    sequence (its cut k >= nx/2), a restart through set_state, and the
    pass count / dto bookkeeping, against the oracle."""
    n = 32
    v = solenoidal_init(n)
    g = oracle_grid(n, nu=0.01, forced=True, eps=0.1, kcut=n // 2)
    ref, t, dto = R.ab2v_run(v, g, STEPS_V)
    ref2, _, _ = R.ab2v_run(v, g, STEPS_V[:2])
    with handle(n, prec, nu=0.01, forced=1, eps=0.1, kcut=n // 2) as h:
        h.set_state(*v)
        for dt in STEPS_V:
            h.ab2v_pass(dt)
        out = h.get_state()
        npass, hdto = h.ab2v_state()
        h.set_state(*v)
        assert h.ab2v_state()[0] == 0
        for dt in STEPS_V[:2]:
            h.ab2v_pass(dt)
        out2 = h.get_state()
    assert npass == len(STEPS_V) and abs(hdto - dto) < 1e-15
    assert rel_l2(out, ref) < TOL[prec]
    assert rel_l2(out2, ref2) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("model", ["smag", "dynsmag"])
def test_variable_step_ab2_les_matches_oracle(specns_lib, prec, model):
    """spectral_les.f90:199-316: the variable-step IF-AB2 with the SGS
    divergence in its right-hand side; with dynsmag the coefficient is
    refreshed on passes 0, 1 and 11 of 12 (spectral_les.f90:140,205-208)."""
    n = 32
    v = solenoidal_init(n)
    sgs = {"smag": S.SC_SGS_SMAG, "dynsmag": S.SC_SGS_DYNSMAG}[model]
    steps = (STEPS_V * 2)[:12] if model == "dynsmag" else STEPS_V
    g = oracle_grid(n, nu=1e-3, forced=True, eps=0.1, sgs=model, c1=0.0289)
    ref, _, _ = R.ab2v_run(v, g, steps)
    with handle(n, prec, nu=1e-3, forced=1, eps=0.1, sgs=sgs, c1=0.0289) as h:
        h.set_state(*v)
        for dt in steps:
            h.ab2v_pass(dt)
        out = h.get_state()
    assert rel_l2(out, ref) < (1e-11 if prec == S.SC_FP64 else 2e-5)


@pytest.mark.parametrize("prec", PRECS)
def test_rotating_scalar_solver_matches_oracle(specns_lib, prec):
    """Five passes of the rotating solver with its passive scalar
    (spectral_rot_dns_scalar_ft.f90:203-291), velocity and scalar forcing on,
    against the oracle; the scalar round-trips through set/get."""
    n, om, pr = 32, 5.0, 0.7
    v = solenoidal_init(n)
    g = oracle_grid(n, nu=0.01, dt=2e-3, forced=True, eps=0.1)
    phi = R.dealiasing(hermitian_fields((n, n, n), 7, ncomp=1)[0], g.k2)
    ref_v, ref_phi, _, _ = R.rot_scalar_run(v, phi, g, 5, om, 1.0, 2.5, pr, True, 0.05)
    with handle(n, prec, nu=0.01, dt=2e-3, forced=1, eps=0.1) as h:
        h.set_state(*v)
        h.set_scalar(phi)
        assert rel_l2(h.get_scalar(), phi) < (1e-15 if prec == S.SC_FP64 else 1e-7)
        h.rot_scalar_steps(5, om=om, fk1=1.0, fk2=2.5, pr=pr, scalarforced=True, epsphi=0.05)
        out_v, out_phi = h.get_state(), h.get_scalar()
    assert rel_l2(out_v, ref_v) < TOL[prec]
    assert rel_l2(out_phi, ref_phi) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("fk1,fk2", [(0.0, 2.5), (1.0, 2.5), (2.0, 5.0)])
def test_forcephi_and_forcephi_rot(specns_lib, prec, fk1, fk2):
    """The passive scalar's forcing (forcephi.f90 on k2 < fk2^2,
    forcephi_rot.f90 on fk1^2 <= k2 < fk2^2) against the oracle."""
    shape = (16, 16, 16)
    phi = hermitian_fields(shape, 8, ncomp=1)[0]
    w = complex_noise(shape, 9, ncomp=1)[0]
    _, _, _, k2 = R.wavenumber(*shape)
    ref = R.forcephi(phi, w, k2, fk2, 0.05)
    ref_rot = R.forcephi_rot(phi, w, k2, fk1, fk2, 0.05)
    (pp,) = cast([phi], prec)
    (ww,) = cast([w], prec)
    S.forcephi(pp, ww, fk2, 0.05)
    assert rel_l2(ww, ref) < TOL[prec]
    assert np.array_equal(pp, cast([phi], prec)[0])      # phi is read only
    (ww,) = cast([w], prec)
    S.forcephi_rot(pp, ww, fk1, fk2, 0.05)
    assert rel_l2(ww, ref_rot) < TOL[prec]
    # the forcing changes w by far more than the tolerance (an identity would fail)
    assert rel_l2(ref, w) > 10 * TOL[prec]


@pytest.mark.parametrize("prec,dtype,real,tol", [("dp", np.complex128, C.c_double, 1e-12),
                                                  ("sp", np.complex64, C.c_float, 1e-5)])
def test_f77_forcephi(specns_lib, prec, dtype, real, tol):
    """forcephi_(phi,wphi,k2,lx1,ly,lz,fkmax,epsphi) and
    forcephi_rot_(phi,wphi,k2,lx1,ly,lz,fk1,fk2,epsphi)."""
    f = _lib.load_f77(prec)
    n = 16
    phi = hermitian_fields((n, n, n), 44, ncomp=1)[0]
    w = hermitian_fields((n, n, n), 45, ncomp=1)[0]
    _, _, _, k2 = R.wavenumber(n, n, n)
    ref = R.forcephi(phi, w, k2, 2.5, 0.05)
    ref_rot = R.forcephi_rot(phi, w, k2, 1.0, 2.5, 0.05)
    k2r = fresh(k2, np.float64 if prec == "dp" else np.float32)
    pp = fresh(phi, dtype)
    ww = fresh(w, dtype)
    f.forcephi_(pp.ctypes.data_as(C.c_void_p), ww.ctypes.data_as(C.c_void_p), k2r.ctypes.data_as(C.c_void_p),
                *ref_int(n // 2 + 1, n, n), C.byref(real(2.5)), C.byref(real(0.05)))
    assert rel_l2(ww, ref) < tol
    ww = fresh(w, dtype)
    f.forcephi_rot_(pp.ctypes.data_as(C.c_void_p), ww.ctypes.data_as(C.c_void_p), k2r.ctypes.data_as(C.c_void_p),
                    *ref_int(n // 2 + 1, n, n), C.byref(real(1.0)), C.byref(real(2.5)), C.byref(real(0.05)))
    assert rel_l2(ww, ref_rot) < tol
    assert rel_l2(ref, w) > 10 * tol


@pytest.mark.parametrize("prec", PRECS)
def test_schemes_against_committed_golden_fixtures(specns_lib, prec):
    """tests/golden/schemes16.npz: the rotating solver, its passive scalar and
    the variable-step IF-AB2 from the seeded 16^3 field."""
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "schemes16.npz"))
    n, nu, dt = int(d["n"]), float(d["nu"]), float(d["dt"])
    v0 = list(d["v0"])
    with handle(n, prec, nu=nu, dt=dt, forced=1, eps=0.1) as h:
        h.set_state(*v0)
        h.rot_steps(5, om=5.0, fk1=1.0, fk2=2.5)
        assert rel_l2(h.get_state(), list(d["v_rot5"])) < TOL[prec]
        h.set_state(*v0)
        h.set_scalar(d["phi0"])
        h.rot_scalar_steps(5, om=5.0, fk1=1.0, fk2=2.5, pr=0.7, scalarforced=True, epsphi=0.05)
        assert rel_l2(h.get_state(), list(d["v_rs5"])) < TOL[prec]
        assert rel_l2(h.get_scalar(), d["phi_rs5"]) < TOL[prec]
    with handle(n, prec, nu=nu, forced=1, eps=0.1, kcut=n // 2) as h:
        h.set_state(*v0)
        for s in d["steps_v"]:
            h.ab2v_pass(float(s))
        assert rel_l2(h.get_state(), list(d["v_ab2v"])) < TOL[prec]
    with handle(n, prec, nu=nu, forced=1, eps=0.1) as h:
        h.set_state(*v0)
        h.set_scalar(R.symmetrize3d(d["phi0"]))
        for s in d["steps_v"]:
            h.ab2v_scalar_pass(float(s), pr=0.7, scalarforced=True, meangrad=0.3)
        assert rel_l2(h.get_state(), list(d["v_vs"])) < TOL[prec]
        assert rel_l2(h.get_scalar(), d["phi_vs"]) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_hermitianize(specns_lib, prec):
    """hermitianize.f90 (sc_hermitianize and the hermitianize_ shim) against
    the oracle on a field with no symmetry."""
    n = 16
    c = complex_noise((n, n, n), 12, ncomp=1)[0]
    ref = R.hermitianize(c)
    # the copy changes the field: a test of the identity would pass otherwise
    assert rel_l2(ref, c) > 0.1
    (cc,) = cast([c], prec)
    S.hermitianize(cc)
    assert rel_l2(cc, ref) < TOL[prec]
    f = _lib.load_f77("dp" if prec == S.SC_FP64 else "sp")
    (cc,) = cast([c], prec)
    f.hermitianize_(cc.ctypes.data_as(C.c_void_p), *ref_int(n // 2 + 1, n, n))
    assert rel_l2(cc, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_outputphi_inputphi_files_and_round_trip(specns_lib, prec, tmp_path):
    """sc_outputphi / sc_inputphi: the scalar as outputphi.f90 writes it
    (phi<n>.dat, one Fortran unformatted record of complex(sp)
    (nx/2+1, ny, nz)), bit for bit, and back, also through a file of the
    other precision."""
    import os
    from oracle import fortran_record as FR
    n = 16
    phi = hermitian_fields((n, n, n), 13, ncomp=1)[0]
    dt = np.complex128 if prec == S.SC_FP64 else np.complex64
    with handle(n, prec) as h:
        h.set_scalar(phi)
        ref = h.get_scalar()
        h.outputphi(tmp_path, 4)
        raw = open(os.path.join(tmp_path, "phi4.dat"), "rb").read()
        assert np.array_equal(np.frombuffer(FR.read_record(raw), dtype=dt).reshape(ref.shape), ref)
        h.set_scalar(np.zeros_like(ref))
        h.inputphi(tmp_path, 4)
        assert np.array_equal(h.get_scalar(), ref)
        other = S.SC_FP32 if prec == S.SC_FP64 else S.SC_FP64
        h.outputphi(tmp_path, 5, file_precision=other)
        h.inputphi(tmp_path, 5, file_precision=other)
        assert rel_l2(h.get_scalar(), ref) < (1e-7 if prec == S.SC_FP64 else 1e-15)
        with pytest.raises(S.SpecNSError):
            h.inputphi(tmp_path, 99)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("history", ["as_written", "rhs"])
def test_variable_step_scalar_matches_oracle(specns_lib, prec, history):
    """Passes of spectral_dns_scalar.f90's variable-step IF-AB2 with the
    passive scalar, mean-gradient forcing on, both scalar histories, against
    the oracle."""
    n = 32
    v = solenoidal_init(n)
    g = oracle_grid(n, nu=0.01, forced=True, eps=0.1)
    phi = R.symmetrize3d(hermitian_fields((n, n, n), 7, ncomp=1)[0])
    ref_v, ref_phi, _, _ = R.ab2v_scalar_run(v, phi, g, STEPS_V, 0.7, True, 0.3, history=history)
    with handle(n, prec, nu=0.01, forced=1, eps=0.1) as h:
        h.set_state(*v)
        h.set_scalar(phi)
        for dt in STEPS_V:
            h.ab2v_scalar_pass(dt, pr=0.7, scalarforced=True, meangrad=0.3, history_rhs=history == "rhs")
        out_v, out_phi = h.get_state(), h.get_scalar()
    assert rel_l2(out_v, ref_v) < TOL[prec]
    assert rel_l2(out_phi, ref_phi) < TOL[prec]
