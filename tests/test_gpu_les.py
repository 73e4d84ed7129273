"""GPU parity of the LES right-hand sides and steps (Smagorinsky, dynamic
Smagorinsky) against the FP64 oracle."""
import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import spectral_ref as R
from _util import hermitian_fields, rel_l2, solenoidal_init

pytestmark = pytest.mark.gpu

PRECS = [S.SC_FP64, S.SC_FP32]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("model", ["smag", "dynsmag"])
def test_les_rhs_and_steps(specns_lib, prec, model):
    n = 32
    v = solenoidal_init(n)
    sgs = S.SC_SGS_SMAG if model == "smag" else S.SC_SGS_DYNSMAG
    g = R.Grid(R.Params(nx=n, nu=1e-3, dt=1e-3, sgs=model, c1=0.0289))
    st = {"cs2": 0.0, "update": True}
    ref_w = R.ratesdudt(v, g, dict(st))
    p = S.default_params(n, prec, nu=1e-3, dt=1e-3, sgs=sgs, c1=0.0289)
    tol = 1e-12 if prec == S.SC_FP64 else 1e-5
    with S.SpectralNS(p) as h:
        h.set_state(*v)
        w = h.rhs()
        assert rel_l2(w, ref_w) < tol
        h.set_state(*v)
        h.rk4_steps(3)
        out = h.get_state()
    ref = R.rk4_run(v, g, 3, sgs_state={"cs2": 0.0, "update": True})
    assert rel_l2(out, ref) < (1e-11 if prec == S.SC_FP64 else 1e-5)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("nx", [128, 256])
@pytest.mark.parametrize("model", ["smag", "dynsmag"])
def test_les_rhs_long_rows(specns_lib, prec, nx, model, monkeypatch):
    """x rows of 64 and 128 complex points, the lengths of the warp-per-row
    x-pass: the LES right-hand side through it (default) and through the
    block x-pass (SPECNS_NO_XWARP=1) against the oracle, on a flat grid
    (ny = nz = 16); then two steps through the captured step graph."""
    ny = nz = 16
    v = hermitian_fields((nx, ny, nz), 71, kcut=2 * (nx // 2) / 3)
    sgs = S.SC_SGS_SMAG if model == "smag" else S.SC_SGS_DYNSMAG
    g = R.Grid(R.Params(nx=nx, ny=ny, nz=nz, nu=1e-3, dt=1e-3, sgs=model, c1=0.0289))
    ref_w = R.ratesdudt(v, g, {"cs2": 0.0, "update": True})
    ref = R.rk4_run(v, g, 2, sgs_state={"cs2": 0.0, "update": True})
    tol = 1e-12 if prec == S.SC_FP64 else 1e-5
    for env in ("0", "1"):
        monkeypatch.setenv("SPECNS_NO_XWARP", env)
        p = S.default_params(nx, prec, nu=1e-3, dt=1e-3, sgs=sgs, c1=0.0289, ny=ny, nz=nz)
        with S.SpectralNS(p) as h:
            h.set_state(*v)
            assert rel_l2(h.rhs(), ref_w) < tol
            h.set_state(*v)
            h.rk4_steps(2)
            assert rel_l2(h.get_state(), ref) < (1e-11 if prec == S.SC_FP64 else 1e-5)
