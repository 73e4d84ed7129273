"""GPU parity of the reference-signature operators against the FP64 oracle.

Tolerances (relative L2 over all output fields): FP64 mode 1e-12, FP32 mode
1e-5 (the bound the FP32-bulk mode is specified to), except where noted.
"""
import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import spectral_ref as R
from _util import complex_noise, fresh, hermitian_fields, rel_l2

pytestmark = pytest.mark.gpu

PRECS = [S.SC_FP64, S.SC_FP32]
TOL = {S.SC_FP64: 1e-12, S.SC_FP32: 1e-5}
DT = {S.SC_FP64: np.complex128, S.SC_FP32: np.complex64}
SHAPES = [(8, 8, 8), (16, 16, 16), (32, 32, 32), (64, 64, 64), (32, 16, 8), (16, 64, 32)]


def cast(fields, prec):
    return [fresh(a, DT[prec]) for a in fields]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("shape", SHAPES)
def test_convec_dns(specns_lib, prec, shape):
    nx, ny, nz = shape
    v = hermitian_fields(shape, 11)
    kx, ky, kz, _ = R.wavenumber(nx, ny, nz)
    w = list(R.vorticity(*v, kx, ky, kz))
    ref = R.convec_dns(*v, *w, nx)
    vv, ww = cast(v, prec), cast(w, prec)
    S.convec_dns(*vv, *ww)
    assert rel_l2(ww, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_convec_dns_roberts_flow_is_beltrami(specns_lib, prec):
    """robertsflow.f90:23-25: w = sqrt(2) u, so the Lamb vector vanishes."""
    n = 32
    x = np.arange(n) * 2 * np.pi / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    u = [np.sin(X) * np.cos(Y), -np.cos(X) * np.sin(Y), np.sqrt(2) * np.sin(X) * np.sin(Y)]
    v = [R.r2c(a) / n ** 3 for a in u]
    kx, ky, kz, _ = R.wavenumber(n, n, n)
    w = list(R.vorticity(*v, kx, ky, kz))
    vv, ww = cast(v, prec), cast(w, prec)
    S.convec_dns(*vv, *ww)
    scale = max(np.abs(a).max() for a in v)
    assert max(np.abs(a).max() for a in ww) < (1e-14 if prec == S.SC_FP64 else 1e-6) * scale


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 16, 8)])
def test_projection(specns_lib, prec, shape):
    nx, ny, nz = shape
    v = complex_noise(shape, 3)
    kx, ky, kz, _ = R.wavenumber(nx, ny, nz)
    ref = R.projection(*v, kx, ky, kz)
    vv = cast(v, prec)
    S.projection(*vv)
    assert rel_l2(vv, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("shape", [(16, 16, 16), (8, 32, 16)])
def test_symmetrize_and_dealiasing(specns_lib, prec, shape):
    nx, ny, nz = shape
    c = complex_noise(shape, 4, 1)[0]
    _, _, _, k2 = R.wavenumber(nx, ny, nz)
    ref = R.symmetrize3d(c)
    cc = cast([c], prec)[0]
    S.symmetrize(cc)
    assert rel_l2(cc, ref) < TOL[prec]
    assert np.array_equal(cc == 0, ref == 0)
    ref2 = R.dealiasing(c, k2)
    cc = cast([c], prec)[0]
    S.dealiasing(cc)
    assert rel_l2(cc, ref2) < TOL[prec]
    assert np.array_equal(cc == 0, ref2 == 0)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("fkmax", [2.5, 4.0])
def test_force(specns_lib, prec, fkmax):
    shape = (16, 16, 16)
    v = hermitian_fields(shape, 5)
    w = complex_noise(shape, 6)
    _, _, _, k2 = R.wavenumber(*shape)
    ref = R.force(*w, *v, k2, fkmax, 0.1)
    ww, vv = cast(w, prec), cast(v, prec)
    S.force(*ww, *vv, fkmax, 0.1)
    assert rel_l2(ww, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", [16, 32])
def test_smag(specns_lib, prec, n):
    v = hermitian_fields((n, n, n), 7, kcut=2 * (n // 2) / 3)
    kx, ky, kz, _ = R.wavenumber(n, n, n)
    delta = R.PI_REF / (2 * (n // 2) / 3)
    ref = R.smag(*v, kx, ky, kz, n, delta, 0.0289)
    t = S.smag(*cast(v, prec), delta, 0.0289)
    assert rel_l2(t, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_dynsmag(specns_lib, prec):
    n = 32
    kcut = 2 * (n // 2) / 3
    v = hermitian_fields((n, n, n), 8, kcut=kcut)
    kx, ky, kz, k2 = R.wavenumber(n, n, n)
    delta = R.PI_REF / kcut
    k_test = kcut / 2
    g = R.test_filter(k2, k_test)
    ref, mm, lm, cs2 = R.dynsmag(*v, kx, ky, kz, g, n, delta, 2 * delta, True, 0.0)
    t, mm_g, lm_g, cs2_g = S.dynsmag(*cast(v, prec), k_test, delta, 2 * delta, True)
    tol = 1e-11 if prec == S.SC_FP64 else 1e-4
    assert abs(cs2_g - cs2) < tol * abs(cs2)
    assert abs(mm_g - mm) < tol * abs(mm) and abs(lm_g - lm) < tol * abs(lm)
    assert rel_l2(t, ref) < tol
    # non-update branch reuses the coefficient (dynsmag.f90:196-232)
    ref2, _, _, _ = R.dynsmag(*v, kx, ky, kz, g, n, delta, 2 * delta, False, 0.05)
    t2, _, _, c2 = S.dynsmag(*cast(v, prec), k_test, delta, 2 * delta, False, 0.05)
    assert c2 == 0.05 and rel_l2(t2, ref2) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 16, 8), (128, 32, 16)])
def test_convecphi_dns(specns_lib, prec, shape):
    """Passive-scalar flux divergence i k . (u phi)^ / N^3 (convecphi_dns.f90)
    against the oracle; (128, 32, 16) takes the warp x-pass for the c2r."""
    nx, ny, nz = shape
    v = hermitian_fields(shape, 21)
    phi = hermitian_fields(shape, 22, ncomp=1)[0]
    ref = R.convecphi_dns(*v, phi, nx)
    vv = cast(v, prec)
    pp = cast([phi], prec)[0]
    out = np.zeros_like(pp)
    S.convecphi_dns(*vv, pp, out, nx)
    assert rel_l2(out, ref) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("fk12,fk22", [(0.0, 6.25), (4.0, 16.0), (9.0, 40.0)])
def test_force_rot(specns_lib, prec, fk12, fk22):
    """Shell-band forcing of the rotating solver (force_rot.f90) against the
    oracle, with the build's tiny (single or double) in the normalisation."""
    shape = (16, 16, 16)
    v = hermitian_fields(shape, 5)
    w = complex_noise(shape, 6)
    _, _, _, k2 = R.wavenumber(*shape)
    tiny = R.MYTINY_SP if prec == S.SC_FP32 else R.MYTINY_DP
    ref = R.force_rot(*w, *v, k2, fk12, fk22, 0.1, tiny)
    ww, vv = cast(w, prec), cast(v, prec)
    S.force_rot(*ww, *vv, fk12, fk22, 0.1)
    assert rel_l2(ww, ref) < TOL[prec]


@pytest.mark.parametrize("prec,tol", [(S.SC_FP64, 1e-12), (S.SC_FP32, 1e-5)])
@pytest.mark.parametrize("shape", [(32, 32, 32), (128, 16, 32)])
def test_skewness_and_enstrophy(specns_lib, prec, tol, shape):
    """Post-processing of skewness.f90 and enstrophy.f90 against the oracle:
    the derivative skewness (a scalar) and the physical enstrophy density."""
    nx = shape[0]
    v = hermitian_fields(shape, 51, kcut=2 * (nx // 2) / 3)
    vv = cast(v, prec)
    s = S.skewness(vv[0], nx)
    s_ref = R.skewness(v[0], nx)
    assert abs(s - s_ref) < tol * max(1.0, abs(s_ref)) * 10
    e = S.enstrophy(*vv, nx)
    e_ref = R.enstrophy_field(*v, nx)
    assert e.shape == e_ref.shape
    assert np.sqrt(np.sum((e - e_ref) ** 2) / np.sum(e_ref ** 2)) < tol * 10
