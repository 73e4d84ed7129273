"""GPU parity of the LES right-hand sides and steps (Smagorinsky, dynamic
Smagorinsky) against the FP64 oracle."""
import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import spectral_ref as R
from _util import rel_l2, solenoidal_init

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
