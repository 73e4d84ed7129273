"""Parity at the sizes of the benchmarked configurations.

* Forced DNS at 512^3 (nu = 1.5e-3, dt = 5e-4, the ran1 seed-1 field with
  E(k) ~ k^4 exp(-2 (k/4)^2), energy 0.5): one plain-FP64 step against the
  oracle's rk4_step (dns-deform.f90:160-237), relative L2 <= 1e-12 over every
  spectral coefficient, and the FP32-bulk step against the FP64 step after 1
  and 10 steps, relative L2 <= 1e-5 over every coefficient, with the shell
  spectrum E(k), the dissipation rate and max |k . v| (FP64 reductions).
* Forced DNS at 128^3 (nu = 0.01, dt = 2e-3): every coefficient after 10
  steps against the oracle (FP64 <= 1e-12, FP32 <= 1e-5, relative L2 and
  max norm).
* LES at 256^3 (nu = 1e-4, dt = 1e-3, c1 = 0.17^2, seeded k^(-5/3) field on
  2 <= k <= 85): two steps of Smagorinsky and of dynamic Smagorinsky
  (coefficient refreshed on step 0) against the oracle (FP64 <= 1e-11, FP32
  <= 2e-5 Smagorinsky, <= 1e-4 dynamic, as the operator tests).
* Adjoint at 256^3, T = 200 steps, checkpoints every K = 20: the FP64
  gradient of the shell-8..16 enstrophy against central differences along
  seeded solenoidal directions (step 1e-4 relative, FP64 forward), <= 1e-6,
  and the FP32 gradient against the FP64 one.

The oracle runs on every host core (scipy.fft workers); these cases take
tens of seconds each.
"""
import os

import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import spectral_ref as R
from _util import rel_l2

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

U0 = 1.0 / np.sqrt(3.0)


@pytest.fixture(autouse=True)
def oracle_threads():
    old = R.WORKERS
    R.WORKERS = len(os.sched_getaffinity(0))
    yield
    R.WORKERS = old


def handle(n, prec, **kw):
    return S.SpectralNS(S.default_params(n, prec, **kw))


def diag_ref(v, g, nu):
    return {"energy": R.energy(v), "dissipation": R.dissipation(v, g.k2, nu),
            "max_div": R.max_divergence(v, g.kx, g.ky, g.kz)}, R.spectrum(v, g.k2, g.p.nx)


C2 = dict(nu=1.5e-3, dt=5e-4, eps=0.1, fkmax=2.5)


def test_c2_512_fp64_step_matches_oracle(specns_lib):
    n = 512
    with handle(n, S.SC_FP64, **C2) as h:
        h.init_field(seed=1, akp=4.0, u0=U0)
        v0 = h.get_state()
        h.rk4_steps(1)
        v1 = h.get_state()
        d, eks = h.diagnostics()
    g = R.Grid(R.Params(nx=n, **C2))
    ref = R.rk4_step(v0, g)
    del v0
    assert rel_l2(v1, ref) <= 1e-12
    dr, ekr = diag_ref(ref, g, C2["nu"])
    assert abs(d["energy"] - dr["energy"]) <= 1e-12 * dr["energy"]
    assert abs(d["dissipation"] - dr["dissipation"]) <= 1e-12 * dr["dissipation"]
    assert abs(d["max_div"] - dr["max_div"]) <= 1e-12 * np.max(np.abs(ref[0]))
    m = ekr > 1e-12 * ekr.sum()
    assert np.max(np.abs(eks[m] - ekr[m]) / ekr[m]) <= 1e-10


def test_c2_512_fp32_against_fp64_after_1_and_10_steps(specns_lib):
    n = 512
    g = R.Grid(R.Params(nx=n, **C2))
    kmax = np.sqrt(float(g.k2.max()))
    with handle(n, S.SC_FP64, **C2) as h64, handle(n, S.SC_FP32, **C2) as h32:
        h64.init_field(seed=1, akp=4.0, u0=U0)
        h32.set_state(*h64.get_state())
        done = 0
        for target in (1, 10):
            h64.rk4_steps(target - done)
            h32.rk4_steps(target - done)
            done = target
            v64, v32 = h64.get_state(), h32.get_state()
            err = rel_l2(v32, v64)
            assert err <= 1e-5, (target, err)
            d64, e64 = h64.diagnostics()
            d32, e32 = h32.diagnostics()
            # shells holding more than 1e-8 of the energy (the rest is round-off)
            m = e64 > 1e-8 * e64.sum()
            assert np.max(np.abs(e32[m] - e64[m]) / e64[m]) <= 1e-5, target
            assert abs(d32["dissipation"] - d64["dissipation"]) <= 1e-5 * d64["dissipation"]
            assert abs(d32["energy"] - d64["energy"]) <= 1e-6 * d64["energy"]
            # the FP32 field stays divergence-free to FP32 round-off of |k||v|
            vmax = max(float(np.max(np.abs(a))) for a in v64)
            assert d32["max_div"] <= 1e-5 * kmax * vmax
            assert d64["max_div"] <= 1e-13 * kmax * vmax


@pytest.mark.parametrize("prec,tol", [(S.SC_FP64, 1e-12), (S.SC_FP32, 1e-5)])
def test_c1_128_every_coefficient_after_10_steps(specns_lib, prec, tol):
    n = 128
    g = R.Grid(R.Params(nx=n, nu=0.01, dt=2e-3))
    with handle(n, S.SC_FP64) as h:
        h.init_field(seed=1, akp=4.0, u0=U0)
        v0 = h.get_state()
    ref = R.rk4_run(v0, g, 10)
    with handle(n, prec) as h:
        h.set_state(*v0)
        h.rk4_steps(10)
        out = h.get_state()
    assert rel_l2(out, ref) <= tol
    # every coefficient, high wavenumbers included, in the max norm
    vmax = max(float(np.max(np.abs(a))) for a in ref)
    assert max(float(np.max(np.abs(a - b))) for a, b in zip(out, ref)) <= tol * vmax


LES = dict(nu=1e-4, dt=1e-3, c1=0.17 ** 2)


@pytest.mark.parametrize("sgs,tols", [("smag", (1e-11, 2e-5)), ("dynsmag", (1e-11, 1e-4))])
def test_c3_les_256_two_steps_match_oracle(specns_lib, sgs, tols):
    n, steps = 256, 2
    code = S.SC_SGS_SMAG if sgs == "smag" else S.SC_SGS_DYNSMAG
    with handle(n, S.SC_FP64, sgs=code, **LES) as h:
        h.init_field(seed=1, kind=1, u0=U0, kmin=2.0, kmax=85.0)
        v0 = h.get_state()
    g = R.Grid(R.Params(nx=n, sgs=sgs, **LES))
    state = {"cs2": 0.0, "update": True} if sgs == "dynsmag" else None
    ref = R.rk4_run(v0, g, steps, state)
    for prec, tol in zip((S.SC_FP64, S.SC_FP32), tols):
        with handle(n, prec, sgs=code, **LES) as h:
            h.set_state(*v0)
            h.rk4_steps(steps)
            out = h.get_state()
            d, _ = h.diagnostics()
        assert rel_l2(out, ref) <= tol, (prec, rel_l2(out, ref))
        if state is not None:
            assert abs(d["cs2"] - state["cs2"]) <= 10 * tol * abs(state["cs2"])


def solenoidal_direction(n, rng):
    kx, ky, kz, k2 = R.wavenumber(n, n, n)
    d = [R.r2c(rng.standard_normal((n, n, n))) / n ** 3 for _ in range(3)]
    d = list(R.projection(*d, kx, ky, kz))
    d = [R.symmetrize3d(a) for a in d]
    return [np.where(k2 >= (2 * (n // 2) / 3) ** 2, 0.0, a) for a in d]


def dot(a, b):
    return sum(float(np.sum((np.conj(x.astype(np.complex128)) * y).real)) for x, y in zip(a, b))


def test_c4_adjoint_256_central_differences(specns_lib):
    n, T, K = 256, 200, 20
    _, _, _, k2 = R.wavenumber(n, n, n)
    grads = {}
    for prec in (S.SC_FP64, S.SC_FP32):
        with handle(n, prec) as h:
            h.init_field(seed=1, akp=4.0, u0=U0)
            if prec == S.SC_FP64:
                v = h.get_state()
            else:
                h.set_state(*v)
            grads[prec] = h.adjoint(T, K, kmin=8, kmax=16)
    J, g64 = grads[S.SC_FP64]
    g32 = grads[S.SC_FP32][1]
    assert abs(grads[S.SC_FP32][0] - J) <= 1e-4 * abs(J)
    assert rel_l2(g32, g64) <= 1e-3
    rng = np.random.default_rng(256)
    vn = np.sqrt(sum(float(np.sum(np.abs(a) ** 2)) for a in v))
    with handle(n, S.SC_FP64) as h:
        def Jof(vv):
            h.set_state(*vv)
            h.rk4_steps(T)
            return R.shell_enstrophy(h.get_state(), k2, 8, 16)

        assert abs(Jof(v) - J) <= 1e-12 * abs(J)
        for _ in range(2):
            d = solenoidal_direction(n, rng)
            dn = np.sqrt(sum(float(np.sum(np.abs(a) ** 2)) for a in d))
            eps = 1e-4 * vn / dn
            fd = (Jof([a + eps * b for a, b in zip(v, d)]) - Jof([a - eps * b for a, b in zip(v, d)])) / (2 * eps)
            assert abs(dot(g64, d) - fd) <= 1e-6 * abs(fd)
            assert abs(dot(g32, d) - fd) <= 1e-3 * abs(fd)
