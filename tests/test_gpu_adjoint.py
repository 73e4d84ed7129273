"""Discrete adjoint of the IF-RK4 step on the GPU.

Checked three ways: against the FP64 oracle adjoint (same discrete map,
rel L2 <= 1e-11), against central finite differences of the GPU forward map
in FP64 (rel <= 1e-7 with a 1e-4 relative step, random non-solenoidal
directions), and FP32 against FP64 (rel L2 <= 1e-4).
"""
import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import spectral_ref as R
from _util import hermitian_fields, rel_l2, solenoidal_init

pytestmark = pytest.mark.gpu


def dot(a, b):
    return sum(float(np.sum((np.conj(x.astype(np.complex128)) * y).real)) for x, y in zip(a, b))


@pytest.mark.parametrize("forced", [1, 0])
def test_adjoint_matches_oracle_fp64(specns_lib, forced):
    n, T, K = 16, 4, 2
    v = solenoidal_init(n)
    g = R.Grid(R.Params(nx=n, nu=0.01, dt=2e-3, forced=bool(forced)))
    ref, Jref = R.adjoint_gradient(v, g, T, kmin=2, kmax=5, checkpoint=K)
    with S.SpectralNS(S.default_params(n, S.SC_FP64, forced=forced)) as h:
        h.set_state(*v)
        J, grad = h.adjoint(T, K, kmin=2, kmax=5)
        v_after = h.get_state()
    assert abs(J - Jref) < 1e-12 * abs(Jref)
    assert rel_l2(grad, ref) < 1e-11
    assert rel_l2(v_after, v) == 0.0   # the state is left at v_0


@pytest.mark.parametrize("n,T,K", [(32, 6, 4)])
def test_adjoint_central_differences_fp64(specns_lib, n, T, K):
    v = solenoidal_init(n)
    _, _, _, k2 = R.wavenumber(n, n, n)
    p = S.default_params(n, S.SC_FP64)
    rng = np.random.default_rng(7)
    with S.SpectralNS(p) as h:
        h.set_state(*v)
        J, grad = h.adjoint(T, K, kmin=8, kmax=16)

        def Jof(vv):
            h.set_state(*vv)
            h.rk4_steps(T)
            return R.shell_enstrophy(h.get_state(), k2, 8, 16)

        assert abs(Jof(v) - J) < 1e-12 * abs(J)
        vn = np.sqrt(sum(float(np.sum(np.abs(a) ** 2)) for a in v))
        for _ in range(3):
            d = [rng.standard_normal(v[0].shape) + 1j * rng.standard_normal(v[0].shape) for _ in range(3)]
            dn = np.sqrt(sum(float(np.sum(np.abs(a) ** 2)) for a in d))
            eps = 1e-4 * vn / dn
            fd = (Jof([a + eps * b for a, b in zip(v, d)]) - Jof([a - eps * b for a, b in zip(v, d)])) / (2 * eps)
            ad = dot(grad, d)
            assert abs(fd - ad) <= 1e-7 * abs(fd)


def test_adjoint_fp32_against_fp64(specns_lib):
    n, T, K = 32, 6, 3
    v = solenoidal_init(n)
    grads = []
    for prec in (S.SC_FP64, S.SC_FP32):
        with S.SpectralNS(S.default_params(n, prec)) as h:
            h.set_state(*v)
            grads.append(h.adjoint(T, K, kmin=8, kmax=16)[1])
    assert rel_l2(grads[1], grads[0]) < 1e-4


def solenoidal_direction(n, rng):
    kx, ky, kz, k2 = R.wavenumber(n, n, n)
    d = [R.r2c(rng.standard_normal((n, n, n))) / n ** 3 for _ in range(3)]
    d = list(R.projection(*d, kx, ky, kz))
    d = [R.symmetrize3d(a) for a in d]
    return [np.where(k2 >= (2 * (n // 2) / 3) ** 2, 0.0, a) for a in d]


@pytest.mark.slow
def test_adjoint_sensitivity_config_128(specns_lib):
    """Gradient of the final-time enstrophy over shells 8..16 after T = 200
    RK4 steps at 128^3, checkpoints every K = 20 steps: the FP64 adjoint
    against central differences along 16 seeded random solenoidal directions
    (step 1e-4 relative, FP64 forward), and the FP32 adjoint against FP64."""
    n, T, K = 128, 200, 20
    v = solenoidal_init(n)
    _, _, _, k2 = R.wavenumber(n, n, n)
    grads = {}
    for prec in (S.SC_FP64, S.SC_FP32):
        with S.SpectralNS(S.default_params(n, prec)) as h:
            h.set_state(*v)
            grads[prec] = h.adjoint(T, K, kmin=8, kmax=16)
    J, g64 = grads[S.SC_FP64]
    g32 = grads[S.SC_FP32][1]
    assert rel_l2(g32, g64) < 1e-3
    rng = np.random.default_rng(2024)
    vn = np.sqrt(sum(float(np.sum(np.abs(a) ** 2)) for a in v))
    worst64 = worst32 = 0.0
    with S.SpectralNS(S.default_params(n, S.SC_FP64)) as h:
        def Jof(vv):
            h.set_state(*vv)
            h.rk4_steps(T)
            return R.shell_enstrophy(h.get_state(), k2, 8, 16)
        for _ in range(16):
            d = solenoidal_direction(n, rng)
            dn = np.sqrt(sum(float(np.sum(np.abs(a) ** 2)) for a in d))
            eps = 1e-4 * vn / dn
            fd = (Jof([a + eps * b for a, b in zip(v, d)]) - Jof([a - eps * b for a, b in zip(v, d)])) / (2 * eps)
            worst64 = max(worst64, abs(dot(g64, d) - fd) / abs(fd))
            worst32 = max(worst32, abs(dot(g32, d) - fd) / abs(fd))
    assert worst64 < 1e-6
    assert worst32 < 1e-3


def test_autograd_function_matches_adjoint_and_fd(specns_lib):
    """The harness's torch.autograd.Function (sc_adjoint_rk4_vjp in backward)
    gives the shell-enstrophy gradient of sc_adjoint_rk4 and matches central
    differences of a generic real loss."""
    torch = pytest.importorskip("torch")
    from _autograd import rk4_steps
    n, T, K = 16, 5, 2
    v = solenoidal_init(n)
    kx, ky, kz, k2 = R.wavenumber(n, n, n)
    shell = np.floor(np.sqrt(k2) + 0.5)
    wk2 = np.where((shell >= 2) & (shell <= 5), k2, 0.0) * np.where(kx == 0, 0.5, 1.0)
    rng = np.random.default_rng(3)
    c = [rng.standard_normal(v[0].shape) + 1j * rng.standard_normal(v[0].shape) for _ in range(3)]
    with S.SpectralNS(S.default_params(n, S.SC_FP64)) as h:
        h.set_state(*v)
        Jad, gad = h.adjoint(T, K, kmin=2, kmax=5)
        vt = [torch.tensor(a, requires_grad=True) for a in v]
        out = rk4_steps(h, T, K, vt)
        J = sum((torch.from_numpy(wk2) * o.abs() ** 2).sum() for o in out)
        J.backward()
        assert abs(J.item() - Jad) < 1e-12 * abs(Jad)
        assert rel_l2([t.grad.numpy() for t in vt], gad) < 1e-12

        def loss(vv):
            h.set_state(*vv)
            h.rk4_steps(T)
            o = h.get_state()
            return sum(float(np.sum((np.conj(ci) * oi).real + 0.25 * np.abs(oi) ** 4)) for ci, oi in zip(c, o))

        vt = [torch.tensor(a, requires_grad=True) for a in v]
        out = rk4_steps(h, T, K, vt)
        L = sum(((torch.from_numpy(ci).conj() * o).real + 0.25 * o.abs() ** 4).sum() for ci, o in zip(c, out))
        L.backward()
        grad = [t.grad.numpy() for t in vt]
        assert abs(L.item() - loss(v)) < 1e-12 * abs(L.item())
        d = [rng.standard_normal(v[0].shape) + 1j * rng.standard_normal(v[0].shape) for _ in range(3)]
        vn = np.sqrt(sum(float(np.sum(np.abs(a) ** 2)) for a in v))
        dn = np.sqrt(sum(float(np.sum(np.abs(a) ** 2)) for a in d))
        eps = 1e-4 * vn / dn
        fd = (loss([a + eps * b for a, b in zip(v, d)]) - loss([a - eps * b for a, b in zip(v, d)])) / (2 * eps)
        assert abs(fd - dot(grad, d)) <= 1e-7 * abs(fd)


def test_adjoint_schedules_agree(specns_lib):
    """Pure checkpointing (budget 0: the last segment recorded by the forward
    sweep, every other one recomputed), one kept segment, and every segment
    kept from the forward sweep give the same J and gradient; the state is
    left at v_0 each time."""
    n, T, K = 16, 7, 3   # segments of 3, 3, 1 steps
    v = solenoidal_init(n)
    nxp = (n // 2 + 1 + 15) // 16 * 16
    fb = 16 * n * n * nxp
    res = []
    with S.SpectralNS(S.default_params(n, S.SC_FP64)) as h:
        for budget, kept in ((0.0, 0), (80.0 * fb, 1), (-1.0, 3)):
            h.set_adjoint_budget(budget)
            h.set_state(*v)
            J, grad = h.adjoint(T, K, kmin=2, kmax=5)
            assert h.adjoint_kept_segments() == kept
            assert rel_l2(h.get_state(), v) == 0.0
            res.append((J, grad))
    for J, grad in res[1:]:
        assert J == res[0][0]
        assert rel_l2(grad, res[0][1]) < 1e-15


@pytest.mark.parametrize("prec,tol", [(S.SC_FP64, 1e-12), (S.SC_FP32, 1e-5)])
def test_adjoint_warp_and_block_xpass_agree(specns_lib, prec, tol, monkeypatch):
    """nx = 128 runs the adjoint product through the warp-per-row x-pass;
    SPECNS_NO_XWARP=1 through the block x-pass.  Same gradient."""
    n, T, K = 128, 2, 1
    v = solenoidal_init(n)
    grads = []
    for env in ("0", "1"):
        monkeypatch.setenv("SPECNS_NO_XWARP", env)
        with S.SpectralNS(S.default_params(n, prec)) as h:
            h.set_state(*v)
            grads.append(h.adjoint(T, K, kmin=8, kmax=16)[1])
    assert rel_l2(grads[0], grads[1]) < tol


def test_adjoint_graph_replay_matches_eager(specns_lib, monkeypatch):
    """The second and later adjoint calls with one schedule replay a captured
    CUDA graph; J and the gradient equal the eager call's bit for bit."""
    n, T, K = 32, 5, 2
    v = solenoidal_init(n)
    res = []
    for env in ("0", "1"):
        monkeypatch.setenv("SPECNS_NO_GRAPH", env)
        with S.SpectralNS(S.default_params(n, S.SC_FP64)) as h:
            for _ in range(3):
                h.set_state(*v)
                res.append(h.adjoint(T, K, kmin=4, kmax=9))
    for J, grad in res[1:]:
        assert J == res[0][0]
        assert rel_l2(grad, res[0][1]) == 0.0


@pytest.mark.parametrize("prec,tol", [(S.SC_FP64, 1e-11), (S.SC_FP32, 1e-4)])
@pytest.mark.parametrize("nz", [256, 512])
def test_adjoint_long_z_matches_oracle(specns_lib, prec, tol, nz):
    """nz = 256 and 512 (the lengths of the two-pass tile transforms, whose
    FP32 form keeps the vorticity's step-1 values in tensor memory): the
    adjoint's z-inverse of the stage inputs runs through them; the gradient
    against the FP64 oracle adjoint, both schedules."""
    nx, ny, T, K = 32, 16, 3, 2
    v = hermitian_fields((nx, ny, nz), 9, kcut=2 * (nx // 2) / 3)
    kx, ky, kz, _ = R.wavenumber(nx, ny, nz)
    v = [R.symmetrize3d(a) for a in R.projection(*v, kx, ky, kz)]
    g = R.Grid(R.Params(nx=nx, ny=ny, nz=nz, nu=0.02, fkmax=6.0))
    ref, Jref = R.adjoint_gradient(v, g, T, kmin=2, kmax=5, checkpoint=K)
    with S.SpectralNS(S.default_params(nx, prec, ny=ny, nz=nz, nu=0.02, fkmax=6.0)) as h:
        for budget in (-1.0, 0.0):
            h.set_adjoint_budget(budget)
            h.set_state(*v)
            J, grad = h.adjoint(T, K, kmin=2, kmax=5)
            assert abs(J - Jref) < tol * abs(Jref)
            assert rel_l2(grad, ref) < tol, (budget, rel_l2(grad, ref))


@pytest.mark.parametrize("prec,tol", [(S.SC_FP64, 1e-11), (S.SC_FP32, 1e-4)])
@pytest.mark.parametrize("nx", [256, 512])
def test_adjoint_long_rows_matches_oracle(specns_lib, prec, tol, nx):
    """nx = 256 and 512 with a small (ny, nz): the adjoint's warp x-pass at
    the row lengths whose FP32 form keeps phi's rows in tensor memory (three
    CTAs per SM at 128-point rows); the gradient against the FP64 oracle
    adjoint, both schedules."""
    ny, nz, T, K = 16, 8, 3, 2
    v = hermitian_fields((nx, ny, nz), 10, kcut=2 * (nz // 2) / 3)
    kx, ky, kz, _ = R.wavenumber(nx, ny, nz)
    v = [R.symmetrize3d(a) for a in R.projection(*v, kx, ky, kz)]
    g = R.Grid(R.Params(nx=nx, ny=ny, nz=nz, nu=0.02, fkmax=3.0))
    ref, Jref = R.adjoint_gradient(v, g, T, kmin=1, kmax=3, checkpoint=K)
    with S.SpectralNS(S.default_params(nx, prec, ny=ny, nz=nz, nu=0.02, fkmax=3.0)) as h:
        for budget in (-1.0, 0.0):
            h.set_adjoint_budget(budget)
            h.set_state(*v)
            J, grad = h.adjoint(T, K, kmin=1, kmax=3)
            assert abs(J - Jref) < tol * abs(Jref)
            assert rel_l2(grad, ref) < tol, (budget, rel_l2(grad, ref))
