"""GPU parity of the right-hand side, the RK4 / AB2 steppers, the seeded
initial field and the FP64 diagnostics against the FP64 oracle.

Parity targets: FP64 mode relative L2 <= 1e-12 after 1 and 10 steps; FP32
bulk mode <= 1e-5 against the FP64 oracle.
"""
import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import spectral_ref as R
from _util import hermitian_fields, rel_l2, solenoidal_init

pytestmark = pytest.mark.gpu

PRECS = [S.SC_FP64, S.SC_FP32]
TOL = {S.SC_FP64: 1e-12, S.SC_FP32: 1e-5}


def handle(n, prec, **kw):
    p = S.default_params(n, prec, **kw)
    return S.SpectralNS(p)


def oracle_grid(n, **kw):
    return R.Grid(R.Params(nx=n, **kw))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [16, 32])
def test_init_field_matches_oracle(specns_lib, prec, n):
    ref = solenoidal_init(n)
    with handle(n, prec) as h:
        h.init_field(seed=1, akp=4.0, u0=1 / np.sqrt(3))
        v = h.get_state()
    assert rel_l2(v, ref) < (1e-13 if prec == S.SC_FP64 else 1e-6)
    assert abs(R.energy(v) - 0.5) < (1e-13 if prec == S.SC_FP64 else 1e-6)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [16, 32])
def test_rhs_matches_ratesdudt(specns_lib, prec, n):
    v = solenoidal_init(n)
    g = oracle_grid(n, nu=0.01, dt=2e-3)
    ref = R.ratesdudt(v, g)
    with handle(n, prec) as h:
        h.set_state(*v)
        w = h.rhs()
    assert rel_l2(w, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_rhs_on_unmasked_hermitian_input(specns_lib, prec):
    """Stage inputs carry modes above the 2/3 cut; the RHS must too."""
    n = 16
    v = hermitian_fields((n, n, n), 21)
    g = oracle_grid(n)
    ref = R.ratesdudt(v, g)
    with handle(n, prec) as h:
        h.set_state(*v)
        w = h.rhs()
    assert rel_l2(w, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,steps", [(16, 1), (16, 10), (32, 1), (32, 10), (64, 1)])
def test_rk4_matches_oracle(specns_lib, prec, n, steps):
    v = solenoidal_init(n)
    g = oracle_grid(n, nu=0.01, dt=2e-3)
    ref = R.rk4_run(v, g, steps)
    with handle(n, prec) as h:
        h.set_state(*v)
        h.rk4_steps(steps)
        out = h.get_state()
    assert rel_l2(out, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_rk4_non_cubic_and_unforced(specns_lib, prec):
    nx, ny, nz = 32, 16, 64
    p = S.default_params(nx, prec, ny=ny, nz=nz, forced=0, nu=0.02)
    v = hermitian_fields((nx, ny, nz), 3, kcut=2 * (nx // 2) / 3)
    kx, ky, kz, _ = R.wavenumber(nx, ny, nz)
    v = [R.symmetrize3d(a) for a in R.projection(*v, kx, ky, kz)]
    g = R.Grid(R.Params(nx=nx, ny=ny, nz=nz, nu=0.02, forced=False))
    ref = R.rk4_run(tuple(v), g, 3)
    with S.SpectralNS(p) as h:
        h.set_state(*v)
        h.rk4_steps(3)
        out = h.get_state()
    assert rel_l2(out, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_rk4_mask_rhs_and_step(specns_lib, prec):
    n = 32
    v = solenoidal_init(n)
    g = oracle_grid(n, mask="rhs_and_step")
    ref = R.rk4_run(v, g, 2)
    with handle(n, prec, mask_mode=S.SC_MASK_RHS_AND_STEP) as h:
        h.set_state(*v)
        h.rk4_steps(2)
        out = h.get_state()
    assert rel_l2(out, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_roberts_flow_decays_exactly(specns_lib, prec):
    """Beltrami flow: zero Lamb vector, so IF-RK4 reproduces exp(-2 nu t)."""
    n = 32
    x = np.arange(n) * 2 * np.pi / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    u = [np.sin(X) * np.cos(Y), -np.cos(X) * np.sin(Y), np.sqrt(2) * np.sin(X) * np.sin(Y)]
    v = [R.r2c(a) / n ** 3 for a in u]
    with handle(n, prec, forced=0, nu=0.05, dt=1e-2) as h:
        h.set_state(*v)
        h.rk4_steps(10)
        out = h.get_state()
    ref = [a * np.exp(-2 * 0.05 * 0.1) for a in v]
    assert rel_l2(out, ref) < (1e-13 if prec == S.SC_FP64 else 1e-6)


@pytest.mark.parametrize("prec", PRECS)
def test_diagnostics(specns_lib, prec):
    n = 32
    v = solenoidal_init(n)
    _, _, _, k2 = R.wavenumber(n, n, n)
    kx, ky, kz, _ = R.wavenumber(n, n, n)
    with handle(n, prec) as h:
        h.set_state(*v)
        d, eks = h.diagnostics()
    tol = 1e-12 if prec == S.SC_FP64 else 1e-6
    assert abs(d["energy"] - R.energy(v)) < tol * R.energy(v)
    assert abs(d["dissipation"] - R.dissipation(v, k2, 0.01)) < tol * R.dissipation(v, k2, 0.01)
    ref_eks = R.spectrum(v, k2, n)
    assert np.max(np.abs(eks - ref_eks)) < tol * np.max(ref_eks)
    assert d["max_div"] < (1e-12 if prec == S.SC_FP64 else 1e-5)
    mu = R.max_velocity(v, n)
    assert abs(d["max_u"] - mu) < (1e-12 if prec == S.SC_FP64 else 1e-5) * mu
    assert d["nonfinite"] == 0


@pytest.mark.parametrize("prec", PRECS)
def test_diagnostics_high_wavenumbers(specns_lib, prec):
    """Diagnostics on a 1024 x 64 x 64 grid of white noise: shells up to
    |k| ~ 514, with k^2 = n^2 + n (the last point of shell n) and n^2 + n + 1
    (the first of shell n + 1) on the grid for large n, so the integer shell
    index is checked at its boundaries; energy, dissipation, every shell,
    max |k . v| and max |u| against the oracle."""
    nx, ny, nz = 1024, 64, 64
    v = hermitian_fields((nx, ny, nz), 83)
    kx, ky, kz, k2 = R.wavenumber(nx, ny, nz)
    with handle(nx, prec, ny=ny, nz=nz) as h:
        nu = h.p.nu
        h.set_state(*v)
        d, eks = h.diagnostics()
    tol = 1e-12 if prec == S.SC_FP64 else 1e-6
    assert abs(d["energy"] - R.energy(v)) < tol * R.energy(v)
    assert abs(d["dissipation"] - R.dissipation(v, k2, nu)) < tol * R.dissipation(v, k2, nu)
    ref_eks = R.spectrum(v, k2, nx)
    assert np.max(np.abs(eks - ref_eks)) < tol * np.max(ref_eks)
    md = R.max_divergence(v, kx, ky, kz)
    assert abs(d["max_div"] - md) < (1e-12 if prec == S.SC_FP64 else 1e-5) * md
    mu = R.max_velocity(v, nx)
    assert abs(d["max_u"] - mu) < (1e-12 if prec == S.SC_FP64 else 1e-5) * mu


@pytest.mark.parametrize("prec", PRECS)
def test_ab2_matches_oracle(specns_lib, prec):
    n = 32
    v = solenoidal_init(n)
    g = oracle_grid(n, nu=0.01, dt=2e-3)
    ref, _ = R.ab2_run(v, g, 6)
    with handle(n, prec) as h:
        h.set_state(*v)
        h.ab2_steps(6)
        out = h.get_state()
    assert rel_l2(out, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_against_committed_golden_fixtures(specns_lib, prec):
    import os
    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    d = np.load(os.path.join(gold, "dns16.npz"))
    n = int(d["n"])
    p = dict(nu=float(d["nu"]), dt=float(d["dt"]))
    with handle(n, prec, **p) as h:
        h.init_field(seed=1, akp=4.0, u0=1 / np.sqrt(3))
        assert rel_l2(h.get_state(), list(d["v0"])) < (1e-14 if prec == S.SC_FP64 else 1e-6)
        h.set_state(*d["v0"])
        assert rel_l2(h.rhs(), list(d["w0"])) < TOL[prec]
        h.rk4_steps(1)
        assert rel_l2(h.get_state(), list(d["v1"])) < TOL[prec]
        h.set_state(*d["v0"])
        h.rk4_steps(10)
        assert rel_l2(h.get_state(), list(d["v10"])) < TOL[prec]
        h.set_state(*d["v0"])
        h.ab2_steps(3)
        assert rel_l2(h.get_state(), list(d["vab3"])) < TOL[prec]
    les = np.load(os.path.join(gold, "les16.npz"))
    v0 = [np.ascontiguousarray(a, np.complex128 if prec == S.SC_FP64 else np.complex64) for a in d["v0"]]
    t = S.smag(*v0, float(les["delta"]), 0.0289)
    assert rel_l2(t, list(les["tau_smag"])) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [32, 64])
def test_rk4_pre_tma_kernels_match(specns_lib, prec, n, monkeypatch):
    """SPECNS_NO_TMA=1 selects the register-fed strided passes; both paths
    must give the oracle's answer."""
    monkeypatch.setenv("SPECNS_NO_TMA", "1")
    v = solenoidal_init(n)
    g = oracle_grid(n, nu=0.01, dt=2e-3)
    ref = R.rk4_run(v, g, 2)
    with handle(n, prec) as h:
        h.set_state(*v)
        h.rk4_steps(2)
        out = h.get_state()
    assert rel_l2(out, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [64, 128, 256])
def test_rhs_block_and_warp_xpass_agree(specns_lib, prec, n, monkeypatch):
    """The warp-per-row x-pass (nx = 128..512) and the block x-pass give the
    oracle's right-hand side."""
    v = hermitian_fields((n, n, n), 41)
    g = oracle_grid(n)
    ref = R.ratesdudt(v, g)
    outs = []
    for env in ("0", "1"):
        monkeypatch.setenv("SPECNS_NO_XWARP", env)
        with handle(n, prec) as h:
            h.set_state(*v)
            outs.append(h.rhs())
    for w in outs:
        assert rel_l2(w, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,fkmax", [(64, 2.5), (64, 20.0), (128, 2.5)])
def test_fused_stage_passes_match_oracle(specns_lib, prec, n, fkmax, monkeypatch):
    """Three z-pass arrangements give the oracle's step: RK stages 1-3 with
    zfwd fused into the next stage's five-transform zinv (default), the
    five-transform zinv alone (SPECNS_NO_FUSE=1) and the register-fed zinv
    (SPECNS_NO_ZINV5=1).  fkmax = 20 puts kx tiles other than the first
    inside the forcing band."""
    v = solenoidal_init(n)
    g = oracle_grid(n, nu=0.01, dt=2e-3, fkmax=fkmax)
    ref = R.rk4_run(v, g, 2)
    outs = []
    for nofuse, noz5 in (("0", "0"), ("1", "0"), ("1", "1")):
        monkeypatch.setenv("SPECNS_NO_FUSE", nofuse)
        monkeypatch.setenv("SPECNS_NO_ZINV5", noz5)
        with handle(n, prec, fkmax=fkmax) as h:
            h.set_state(*v)
            h.rk4_steps(2)
            outs.append(h.get_state())
    for o in outs:
        assert rel_l2(o, ref) < TOL[prec]
    for o in outs[1:]:
        assert rel_l2(outs[0], o) < (1e-13 if prec == S.SC_FP64 else 2e-6)


@pytest.mark.parametrize("prec", PRECS)
def test_graph_replay_matches_eager(specns_lib, prec, monkeypatch):
    """sc_rk4_steps replays one captured RK4 step as a CUDA graph; the result
    is bit-identical to launching every kernel (SPECNS_NO_GRAPH=1), across
    repeated calls and a change of dt."""
    n = 32
    v = solenoidal_init(n)
    outs = []
    for env in ("0", "1"):
        monkeypatch.setenv("SPECNS_NO_GRAPH", env)
        with handle(n, prec) as h:
            h.set_state(*v)
            h.rk4_steps(4)
            h.rk4_steps(3)
            h.set_dt(1e-3)
            h.rk4_steps(2)
            outs.append(h.get_state())
    assert rel_l2(outs[0], outs[1]) == 0.0


@pytest.mark.parametrize("prec,tol", [(S.SC_FP64, (1e-12, 1e-12, 1e-11)), (S.SC_FP32, (1e-5, 1e-5, 1e-4))])
def test_c1_forced_dns_128_against_fixture(specns_lib, prec, tol):
    """Forced DNS at 128^3 (nu = 0.01, dt = 2e-3, the seeded ran1 field)
    after 1, 10 and 100 steps against the oracle's committed results
    (tests/golden/c1_128.npz): the wavenumbers |k| <= 6 per axis, and the
    shell spectrum, energy and dissipation (FP64 diagnostics) at step 100."""
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "c1_128.npz"))
    n, km = int(d["n"]), int(d["kmax"])
    idx = np.r_[0:km + 1, n - km:n]

    def block(v):
        return np.stack([a[np.ix_(idx, idx, np.arange(km + 1))] for a in v])

    with handle(n, prec, nu=float(d["nu"]), dt=float(d["dt"])) as h:
        h.init_field(seed=1, akp=4.0, u0=1 / np.sqrt(3))
        done = 0
        for i, target in enumerate((1, 10, 100)):
            h.rk4_steps(target - done)
            done = target
            assert rel_l2(block(h.get_state()), d["v%d" % target]) < tol[i], target
        diag, eks = h.diagnostics()
    ek = d["ek100"]
    m = ek > 1e-10 * ek.sum()
    assert np.max(np.abs(eks[m] - ek[m]) / ek[m]) < 10 * tol[2]
    assert abs(diag["energy"] - float(d["energy100"])) < tol[2] * float(d["energy100"])
    assert abs(diag["dissipation"] - float(d["diss100"])) < tol[2] * float(d["diss100"])


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("nz", [256, 512])
def test_fused_stage_passes_long_z(specns_lib, prec, nz, monkeypatch):
    """nz = 256 and 512 with a small (nx, ny): the z-passes of the fused step
    at the lengths of the two-pass tile transforms (FP32 with the vorticity's
    step-1 values in tensor memory) against the oracle, in all three z-pass
    arrangements, forcing band wide enough to reach kx tiles past the
    first."""
    nx, ny = 32, 16
    v = hermitian_fields((nx, ny, nz), 5, kcut=2 * (nx // 2) / 3)
    kx, ky, kz, _ = R.wavenumber(nx, ny, nz)
    v = [R.symmetrize3d(a) for a in R.projection(*v, kx, ky, kz)]
    g = R.Grid(R.Params(nx=nx, ny=ny, nz=nz, nu=0.02, fkmax=6.0))
    ref = R.rk4_run(tuple(v), g, 2)
    outs = []
    for nofuse, noz5 in (("0", "0"), ("1", "0"), ("1", "1")):
        monkeypatch.setenv("SPECNS_NO_FUSE", nofuse)
        monkeypatch.setenv("SPECNS_NO_ZINV5", noz5)
        with S.SpectralNS(S.default_params(nx, prec, ny=ny, nz=nz, nu=0.02, fkmax=6.0)) as h:
            h.set_state(*v)
            h.rk4_steps(2)
            outs.append(h.get_state())
    for o in outs:
        assert rel_l2(o, ref) < TOL[prec]
    for o in outs[1:]:
        assert rel_l2(outs[0], o) < (1e-13 if prec == S.SC_FP64 else 2e-6)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("nx", [256, 512])
def test_rk4_long_rows(specns_lib, prec, nx):
    """nx = 256 and 512 with a small (ny, nz): the warp x-pass at the row
    lengths whose FP32 form keeps u's rows in tensor memory (and runs three
    CTAs per SM at 128-point rows), two forced RK4 steps against the oracle."""
    ny, nz = 16, 8
    v = hermitian_fields((nx, ny, nz), 12, kcut=2 * (nz // 2) / 3)
    kx, ky, kz, _ = R.wavenumber(nx, ny, nz)
    v = [R.symmetrize3d(a) for a in R.projection(*v, kx, ky, kz)]
    g = R.Grid(R.Params(nx=nx, ny=ny, nz=nz, nu=0.02, fkmax=3.0))
    ref = R.rk4_run(tuple(v), g, 2)
    with S.SpectralNS(S.default_params(nx, prec, ny=ny, nz=nz, nu=0.02, fkmax=3.0)) as h:
        h.set_state(*v)
        h.rk4_steps(2)
        out = h.get_state()
    assert rel_l2(out, ref) < TOL[prec]
