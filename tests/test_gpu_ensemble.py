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


@pytest.mark.parametrize("prec,tol", [(S.SC_FP64, 1e-12), (S.SC_FP32, 1e-5)])
def test_ensemble_matches_oracle(specns_lib, prec, tol):
    dts, nus = zip(*[params(n) for n in SIZES])
    seeds = [-(i + 1) for i in range(len(SIZES))]
    init = [R.initialize2d(n, s) for n, s in zip(SIZES, seeds)]
    outs = {}
    for mode in (0, 1, 2):
        with S.Ensemble2D(SIZES, dts, nus, 0.01, prec) as e:
            e.init(seeds)
            for m, n in enumerate(SIZES):
                assert rel_l2(e.get_member(m), init[m]) < (1e-14 if prec == S.SC_FP64 else 1e-6)
            e.rk4_steps(3, mode)
            outs[mode] = [e.get_member(m) for m in range(len(SIZES))]
            if mode == 0:
                assert e.uses_graph()
    for m, n in enumerate(SIZES):
        p = R.Params2D(n=n, alpha=0.01, nu8=nus[m], dt=dts[m])
        w = init[m]
        for _ in range(3):
            w = R.rk4_step2d(w, p)
        assert rel_l2(outs[0][m], w) < tol, (m, n)
        assert np.array_equal(outs[0][m], outs[1][m]) and np.array_equal(outs[0][m], outs[2][m])


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
