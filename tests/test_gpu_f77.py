"""The Fortran-ABI shims (reference signatures, by-reference arguments)
called the way gfortran would call them, checked against the oracle."""
import ctypes as C

import numpy as np
import pytest

from oracle import spectral_ref as R
from speccodelib_gb300 import _lib
from _util import hermitian_fields, rel_l2

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
    vv = [np.ascontiguousarray(a, dtype) for a in v]
    ww = [np.ascontiguousarray(a, dtype) for a in w]
    f.convec_dns_(*[a.ctypes.data_as(C.c_void_p) for a in vv + ww], *ref_int(n // 2 + 1, n, n, n, n, n))
    assert rel_l2(ww, ref) < tol
    # projection_(vx,vy,vz,kx,ky,kz,lx1,ly,lz)
    ref_p = R.projection(*w, kx, ky, kz)
    ww = [np.ascontiguousarray(a, dtype) for a in w]
    kr = [np.ascontiguousarray(a, np.float64 if prec == "dp" else np.float32) for a in (kx, ky, kz)]
    f.projection_(*[a.ctypes.data_as(C.c_void_p) for a in ww], *[a.ctypes.data_as(C.c_void_p) for a in kr],
                  *ref_int(n // 2 + 1, n, n))
    assert rel_l2(ww, ref_p) < tol
    c = np.ascontiguousarray(w[0], dtype)
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
    vv = [np.ascontiguousarray(a, dtype) for a in v]
    t = [np.zeros_like(vv[0]) for _ in range(6)]
    k3 = [np.ascontiguousarray(np.broadcast_to(a, k2.shape), rdt) for a in
          (kx[None, None, :], ky[None, :, None], kz[:, None, None])]
    gg = np.ascontiguousarray(g, rdt)
    out = [real(0), real(0), real(0)]
    f.dynsmag_(*[a.ctypes.data_as(C.c_void_p) for a in vv + t + k3 + [gg]],
               *ref_int(n // 2 + 1, n, n, n, n, n, n // 2),
               C.byref(real(delta)), C.byref(real(2 * delta)),
               *[C.byref(o) for o in out], C.byref(C.c_int(1)))
    assert abs(out[2].value - cs2) < tol * abs(cs2) * 10
    assert rel_l2(t, ref) < tol * 10
