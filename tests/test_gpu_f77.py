"""The Fortran-ABI shims (reference signatures, by-reference arguments)
called the way gfortran would call them, checked against the oracle."""
import ctypes as C

import numpy as np
import pytest

from oracle import spectral_ref as R
from speccodelib_gb300 import _lib
from _util import fresh, hermitian_fields, rel_l2

pytestmark = pytest.mark.gpu


def ref_int(*xs):
    return [C.byref(C.c_int(x)) for x in xs]


@pytest.mark.parametrize("prec,dtype,real,tol", [("dp", np.complex128, C.c_double, 1e-12),
                                                  ("sp", np.complex64, C.c_float, 1e-5)])
def test_f77_convec_projection_symmetrize(specns_lib, prec, dtype, real, tol):
    f = _lib.load_f77(prec)
    n = 16
    v = hermitian_fields((n, n, n), 31)
    kx, ky, kz, k2 = R.wavenumber(n, n, n)
    w = list(R.vorticity(*v, kx, ky, kz))
    ref = R.convec_dns(*v, *w, n)
    vv = [fresh(a, dtype) for a in v]
    ww = [fresh(a, dtype) for a in w]
    f.convec_dns_(*[a.ctypes.data_as(C.c_void_p) for a in vv + ww], *ref_int(n // 2 + 1, n, n, n, n, n))
    assert rel_l2(ww, ref) < tol
    # projection_(vx,vy,vz,kx,ky,kz,lx1,ly,lz)
    ref_p = R.projection(*w, kx, ky, kz)
    ww = [fresh(a, dtype) for a in w]
    kr = [fresh(a, np.float64 if prec == "dp" else np.float32) for a in (kx, ky, kz)]
    f.projection_(*[a.ctypes.data_as(C.c_void_p) for a in ww], *[a.ctypes.data_as(C.c_void_p) for a in kr],
                  *ref_int(n // 2 + 1, n, n))
    assert rel_l2(ww, ref_p) < tol
    c = fresh(w[0], dtype)
    f.__msymmetrize_MOD_symmetrize3d(c.ctypes.data_as(C.c_void_p), *ref_int(n // 2 + 1, n, n))
    assert rel_l2(c, R.symmetrize3d(w[0])) < tol


@pytest.mark.parametrize("prec,dtype,real,tol", [("dp", np.complex128, C.c_double, 1e-11),
                                                  ("sp", np.complex64, C.c_float, 1e-4)])
def test_f77_dynsmag_recovers_test_filter(specns_lib, prec, dtype, real, tol):
    f = _lib.load_f77(prec)
    n = 32
    kcut = 2 * (n // 2) / 3
    v = hermitian_fields((n, n, n), 32, kcut=kcut)
    kx, ky, kz, k2 = R.wavenumber(n, n, n)
    delta = R.PI_REF / kcut
    g = R.test_filter(k2, kcut / 2)
    ref, mm, lm, cs2 = R.dynsmag(*v, kx, ky, kz, g, n, delta, 2 * delta, True, 0.0)
    rdt = np.float64 if prec == "dp" else np.float32
    vv = [fresh(a, dtype) for a in v]
    t = [np.zeros_like(vv[0]) for _ in range(6)]
    k3 = [fresh(np.broadcast_to(a, k2.shape), rdt) for a in
          (kx[None, None, :], ky[None, :, None], kz[:, None, None])]
    gg = fresh(g, rdt)
    out = [real(0), real(0), real(0)]
    f.dynsmag_(*[a.ctypes.data_as(C.c_void_p) for a in vv + t + k3 + [gg]],
               *ref_int(n // 2 + 1, n, n, n, n, n, n // 2),
               C.byref(real(delta)), C.byref(real(2 * delta)),
               *[C.byref(o) for o in out], C.byref(C.c_int(1)))
    assert abs(out[2].value - cs2) < tol * abs(cs2) * 10
    assert rel_l2(t, ref) < tol * 10


@pytest.mark.parametrize("prec,dtype,real,tol", [("dp", np.complex128, C.c_double, 1e-12),
                                                  ("sp", np.complex64, C.c_float, 1e-5)])
def test_f77_convecphi_and_force_rot(specns_lib, prec, dtype, real, tol):
    """convecphi_dns_(vx,vy,vz,phi,wphi,kx,ky,kz,lx1,ly,lz,nx,ny,nz) and
    force_rot_(wx,wy,wz,vx,vy,vz,k2,lx1,ly,lz,fk12,fk22,eps)."""
    f = _lib.load_f77(prec)
    n = 16
    v = hermitian_fields((n, n, n), 41)
    phi = hermitian_fields((n, n, n), 42, ncomp=1)[0]
    kx, ky, kz, k2 = R.wavenumber(n, n, n)
    rdt = np.float64 if prec == "dp" else np.float32
    vv = [fresh(a, dtype) for a in v]
    pp = fresh(phi, dtype)
    out = np.zeros_like(pp)
    kr = [fresh(a, rdt) for a in (kx, ky, kz)]
    f.convecphi_dns_(*[a.ctypes.data_as(C.c_void_p) for a in vv + [pp, out] + kr], *ref_int(n // 2 + 1, n, n, n, n, n))
    assert rel_l2(out, R.convecphi_dns(*v, phi, n)) < tol
    w = [fresh(a, dtype) for a in hermitian_fields((n, n, n), 43)]
    tiny = R.MYTINY_DP if prec == "dp" else R.MYTINY_SP
    ref = R.force_rot(*[a.astype(np.complex128) for a in w], *v, k2, 4.0, 16.0, 0.1, tiny)
    k2r = fresh(k2, rdt)
    f.force_rot_(*[a.ctypes.data_as(C.c_void_p) for a in w + vv], k2r.ctypes.data_as(C.c_void_p),
                 *ref_int(n // 2 + 1, n, n), C.byref(real(4.0)), C.byref(real(16.0)), C.byref(real(0.1)))
    assert rel_l2(w, ref) < tol


@pytest.mark.parametrize("prec,dtype,real,tol", [("dp", np.complex128, C.c_double, 1e-11),
                                                  ("sp", np.complex64, C.c_float, 1e-4)])
def test_f77_skewness_and_enstrophy(specns_lib, prec, dtype, real, tol):
    """skewness_(ux,kx,s,nx,ny,nz) (s real(sp)) and enstrophy_(...) (always
    double precision, as the reference declares it)."""
    f = _lib.load_f77(prec)
    n = 16
    v = hermitian_fields((n, n, n), 61, kcut=2 * (n // 2) / 3)
    kx, ky, kz, k2 = R.wavenumber(n, n, n)
    u = fresh(v[0], dtype)
    kr = fresh(kx, np.float64 if prec == "dp" else np.float32)
    s = real(0)
    f.skewness_(u.ctypes.data_as(C.c_void_p), kr.ctypes.data_as(C.c_void_p), C.byref(s), *ref_int(n, n, n))
    assert abs(s.value - R.skewness(v[0], n)) < tol * 10
    uu = [fresh(a, np.complex128) for a in v]
    kd = [np.zeros((n, n, n // 2 + 1)) for _ in range(3)]
    e = np.zeros((n, n, n))
    f.enstrophy_(*[a.ctypes.data_as(C.c_void_p) for a in uu + kd + [e]], *ref_int(n // 2 + 1, n, n, n // 2, n, n, n))
    e_ref = R.enstrophy_field(*v, n)
    assert np.sqrt(np.sum((e - e_ref) ** 2) / np.sum(e_ref ** 2)) < 1e-12
