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
from _util import rel_l2, solenoidal_init

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
