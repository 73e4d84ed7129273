"""Batched 2D vorticity ensembles against the FP64 oracle (rhs2d,
rk4_step2d, initialize2d): every member of a mixed-size ensemble after a few
IF-RK4 steps, in all three execution modes (graph, plain, one member at a
time), which must agree bit for bit."""
import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import spectral_ref as R
from _util import rel_l2

pytestmark = pytest.mark.gpu

SIZES = [64, 128, 256, 128, 64]


def params(n):
    kmax = 2.0 * (n // 2) / 3.0
    dt = 0.5 / n
    return dt, 1.0 / (kmax ** 8 * dt)


NVAR = {S.SC_FP32: 6, S.SC_FP64: 2}


def oracle_steps(n, w, dt, nu, steps):
    p = R.Params2D(n=n, alpha=0.01, nu8=nu, dt=dt)
    for _ in range(steps):
        w = R.rk4_step2d(w, p)
    return w


@pytest.mark.parametrize("prec,tol", [(S.SC_FP64, 1e-12), (S.SC_FP32, 1e-5)])
def test_ensemble_matches_oracle(specns_lib, prec, tol):
    """Every compiled launch shape (pinned with set_variant), in all three
    modes; the modes agree bit for bit within a shape."""
    dts, nus = zip(*[params(n) for n in SIZES])
    seeds = [-(i + 1) for i in range(len(SIZES))]
    init = [R.initialize2d(n, s) for n, s in zip(SIZES, seeds)]
    ref = [oracle_steps(n, init[m], dts[m], nus[m], 3) for m, n in enumerate(SIZES)]
    for v in range(NVAR[prec]):
        outs = {}
        for mode in (0, 1, 2):
            with S.Ensemble2D(SIZES, dts, nus, 0.01, prec) as e:
                e.set_variant(v)
                e.init(seeds)
                for m, n in enumerate(SIZES):
                    assert rel_l2(e.get_member(m), init[m]) < (1e-14 if prec == S.SC_FP64 else 1e-6)
                e.rk4_steps(3, mode)
                outs[mode] = [e.get_member(m) for m in range(len(SIZES))]
                if mode == 0:
                    assert e.uses_graph()
                assert e.variant()[0] == v
        for m, n in enumerate(SIZES):
            assert rel_l2(outs[0][m], ref[m]) < tol, (v, m, n)
            assert np.array_equal(outs[0][m], outs[1][m]) and np.array_equal(outs[0][m], outs[2][m])


@pytest.mark.parametrize("prec,tol", [(S.SC_FP64, 1e-12), (S.SC_FP32, 1e-5)])
def test_ensemble_large_members(specns_lib, prec, tol):
    """N = 512 and 1024 members (the 16- and 32-point-per-lane x rows)."""
    sizes = [1024, 512]
    dts, nus = zip(*[params(n) for n in sizes])
    seeds = [-7, -8]
    for v in range(NVAR[prec]):
        with S.Ensemble2D(sizes, dts, nus, 0.01, prec) as e:
            e.set_variant(v)
            e.init(seeds)
            init = [e.get_member(m) for m in range(2)]
            e.rk4_steps(2)
            out = [e.get_member(m) for m in range(2)]
        for m, n in enumerate(sizes):
            w0 = init[m].astype(np.complex128)
            assert rel_l2(w0, R.initialize2d(n, seeds[m])) < (1e-14 if prec == S.SC_FP64 else 1e-6)
            assert rel_l2(out[m], oracle_steps(n, R.initialize2d(n, seeds[m]), dts[m], nus[m], 2)) < tol, (v, n)


def test_ensemble_autotuner(specns_lib):
    """The tuner times every shape, keeps the fastest, and leaves the member
    states as they were; stepping afterwards equals the pinned shape."""
    dts, nus = zip(*[params(n) for n in SIZES])
    seeds = [-(i + 1) for i in range(len(SIZES))]
    with S.Ensemble2D(SIZES, dts, nus, 0.01, S.SC_FP32) as e:
        e.init(seeds)
        before = [e.get_member(m) for m in range(len(SIZES))]
        chosen = e.tune(2)
        v, shape, ms = e.variant()
        assert v == chosen and len(ms) == NVAR[S.SC_FP32] and all(t > 0 for t in ms)
        assert ms[v] == min(ms)
        assert shape["threads"] in (256, 512) and shape["radix"] in (4, 8)
        for m in range(len(SIZES)):
            assert np.array_equal(e.get_member(m), before[m])
        e.rk4_steps(2)
        tuned = [e.get_member(m) for m in range(len(SIZES))]
    with S.Ensemble2D(SIZES, dts, nus, 0.01, S.SC_FP32) as e:
        e.set_variant(chosen)
        e.init(seeds)
        e.rk4_steps(2)
        for m in range(len(SIZES)):
            assert np.array_equal(e.get_member(m), tuned[m])


def test_ensemble_energy_decays_without_forcing(specns_lib):
    n = 128
    dt, nu = params(n)
    with S.Ensemble2D([n, n], [dt, dt], [nu, nu], 0.01, S.SC_FP64) as e:
        e.init([-3, -4])
        e0 = [R.energy2d(e.get_member(m)) for m in range(2)]
        e.rk4_steps(20)
        e1 = [R.energy2d(e.get_member(m)) for m in range(2)]
    assert all(abs(a - 0.5) < 1e-12 for a in e0)
    assert all(b < a for a, b in zip(e0, e1))
