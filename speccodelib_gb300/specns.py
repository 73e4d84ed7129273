"""Host-side mirror of the reference's hot-path interface over the C ABI.

The functions here keep the names, argument meaning and in-place behaviour of
the reference's Fortran subroutines (convec_dns.f90, projection.f90,
force.f90, symmetrize.f90, dealiasing.f90, smag.f90, dynsmag.f90): arrays are
NumPy arrays in the reference's half-complex layout -- shape
``(nz, ny, nx//2 + 1)`` in C order, which is the memory of the Fortran array
``c(lx1, ly, lz)`` -- of dtype complex64 (FP32 mode) or complex128 (FP64
mode), and outputs overwrite the reference's ``intent(inout)`` arguments.

`SpectralNS` wraps the handle API (device-resident state, RK4 / AB2 steps,
diagnostics).  Every call goes through ``libspecns.so``; there is no CPU
fallback, and a missing library raises at import.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib

SC_OK = 0
SC_FP32, SC_FP64 = 0, 1
SC_SGS_NONE, SC_SGS_SMAG, SC_SGS_DYNSMAG = 0, 1, 2
SC_MASK_AFTER_STEP, SC_MASK_RHS_AND_STEP = 0, 1
ERRORS = {1: "SC_ERR_INVALID", 2: "SC_ERR_CUDA", 3: "SC_ERR_NONFINITE",
          4: "SC_ERR_TIMEOUT", 5: "SC_ERR_NOMEM"}


class SpecNSError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, code), msg))
        self.code = code


class Params(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("precision", C.c_int),
                ("nu", C.c_double), ("dt", C.c_double), ("forced", C.c_int),
                ("eps", C.c_double), ("fkmax", C.c_double), ("kcut", C.c_double),
                ("sgs", C.c_int), ("c1", C.c_double), ("delta", C.c_double),
                ("delta_ratio", C.c_double), ("dyn_every", C.c_int), ("mask_mode", C.c_int)]


class Diag(C.Structure):
    _fields_ = [("energy", C.c_double), ("enstrophy", C.c_double), ("dissipation", C.c_double),
                ("max_div", C.c_double), ("max_u", C.c_double), ("nonfinite", C.c_double),
                ("cs2", C.c_double), ("mm", C.c_double), ("lm", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib():
    return _lib.load()


def _check(rc):
    if rc != SC_OK:
        raise SpecNSError(rc, lib().sc_last_error().decode())


def _prec_of(a):
    if a.dtype == np.complex64:
        return SC_FP32
    if a.dtype == np.complex128:
        return SC_FP64
    raise TypeError("arrays must be complex64 (FP32) or complex128 (FP64), got %s" % a.dtype)


def _ptr(a, writable=False):
    if not isinstance(a, np.ndarray) or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous NumPy array in the (nz, ny, nx/2+1) layout")
    if writable and not a.flags.writeable:
        raise TypeError("output array is read-only")
    return C.c_void_p(a.ctypes.data)


def _same(*arrs):
    a0 = arrs[0]
    for a in arrs[1:]:
        if a.shape != a0.shape or a.dtype != a0.dtype:
            raise TypeError("all arrays must share shape and dtype")
    if a0.ndim != 3:
        raise TypeError("expected 3D arrays of shape (nz, ny, nx/2+1)")
    nz, ny, lx1 = a0.shape
    return _prec_of(a0), lx1, ny, nz


# ---------------------------------------------------------------------------
# reference-signature operators
# ---------------------------------------------------------------------------
def convec_dns(vx, vy, vz, wx, wy, wz, nx=None):
    """convec_dns.f90:1 -- w <- spectral Lamb vector of (v, w); in place."""
    prec, lx1, ly, lz = _same(vx, vy, vz, wx, wy, wz)
    nx = nx or 2 * (lx1 - 1)
    _check(lib().sc_convec_dns(prec, _ptr(vx), _ptr(vy), _ptr(vz), _ptr(wx, True), _ptr(wy, True),
                               _ptr(wz, True), lx1, ly, lz, nx, ly, lz))


def projection(vx, vy, vz):
    """projection.f90:2 -- v <- v - k (k.v)/k^2; in place."""
    prec, lx1, ly, lz = _same(vx, vy, vz)
    _check(lib().sc_projection(prec, _ptr(vx, True), _ptr(vy, True), _ptr(vz, True), lx1, ly, lz))


def force(wx, wy, wz, vx, vy, vz, fkmax, eps):
    """force.f90:3 -- w += eps/(2 K_f) v on k2 < fkmax^2; in place on w."""
    prec, lx1, ly, lz = _same(wx, wy, wz, vx, vy, vz)
    _check(lib().sc_force(prec, _ptr(wx, True), _ptr(wy, True), _ptr(wz, True), _ptr(vx), _ptr(vy),
                          _ptr(vz), lx1, ly, lz, C.c_double(fkmax), C.c_double(eps)))



def force_rot(wx, wy, wz, vx, vy, vz, fk12, fk22, eps):
    """force_rot.f90:3 -- w += eps/(2 K + tiny) v on fk12 <= k2 < fk22; in place on w."""
    prec, lx1, ly, lz = _same(wx, wy, wz, vx, vy, vz)
    _check(lib().sc_force_rot(prec, _ptr(wx, True), _ptr(wy, True), _ptr(wz, True), _ptr(vx), _ptr(vy),
                              _ptr(vz), lx1, ly, lz, C.c_double(fk12), C.c_double(fk22), C.c_double(eps)))


def forcephi(phi, wphi, fkmax, epsphi):
    """forcephi.f90:1 -- wphi += epsphi/(2 K) phi on k2 < fkmax^2; in place on wphi."""
    prec, lx1, ly, lz = _same(phi, wphi)
    _check(lib().sc_forcephi(prec, _ptr(phi), _ptr(wphi, True), lx1, ly, lz, C.c_double(fkmax),
                             C.c_double(epsphi)))


def forcephi_rot(phi, wphi, fk1, fk2, epsphi):
    """forcephi_rot.f90:1 -- the same on fk1^2 <= k2 < fk2^2; in place on wphi."""
    prec, lx1, ly, lz = _same(phi, wphi)
    _check(lib().sc_forcephi_rot(prec, _ptr(phi), _ptr(wphi, True), lx1, ly, lz, C.c_double(fk1),
                                 C.c_double(fk2), C.c_double(epsphi)))


def skewness(ux, nx):
    """skewness.f90:1 -- velocity-derivative skewness <d^3>/<d^2>^(3/2), d = du_x/dx."""
    prec, lx1, ly, lz = _same(ux)
    s = C.c_double(0)
    _check(lib().sc_skewness(prec, _ptr(ux), nx, ly, lz, C.byref(s)))
    return s.value


def enstrophy(ux, uy, uz, nx):
    """enstrophy.f90:1 -- 1/2 |curl u|^2 at every physical point, (nz, ny, nx) float64."""
    prec, lx1, ly, lz = _same(ux, uy, uz)
    out = np.zeros((lz, ly, nx), dtype=np.float64)
    _check(lib().sc_enstrophy(prec, _ptr(ux), _ptr(uy), _ptr(uz), _ptr(out, True), lx1, ly, lz, nx, ly, lz))
    return out


def convecphi_dns(vx, vy, vz, phi, wphi, nx):
    """convecphi_dns.f90:1 -- wphi <- i k . (u phi)^ / N^3; writes wphi."""
    prec, lx1, ly, lz = _same(vx, vy, vz, phi, wphi)
    _check(lib().sc_convecphi_dns(prec, _ptr(vx), _ptr(vy), _ptr(vz), _ptr(phi), _ptr(wphi, True),
                                  lx1, ly, lz, nx, ly, lz))

def symmetrize(c):
    """symmetrize.f90:32 (3D) -- in place."""
    prec, lx1, ly, lz = _same(c)
    _check(lib().sc_symmetrize(prec, _ptr(c, True), lx1, ly, lz))


def hermitianize(c):
    """hermitianize.f90:1 -- the kx = 0 conjugate symmetry alone; in place."""
    prec, lx1, ly, lz = _same(c)
    _check(lib().sc_hermitianize(prec, _ptr(c, True), lx1, ly, lz))


def dealiasing(c):
    """dealiasing.f90:2 -- symmetrize + zero k2 >= ly^2/9; in place."""
    prec, lx1, ly, lz = _same(c)
    _check(lib().sc_dealiasing(prec, _ptr(c, True), lx1, ly, lz))


def smag(vx, vy, vz, delta, c1=0.026):
    """smag.f90:1 -- returns [t11, t12, t13, t22, t23, t33] (spectral)."""
    prec, lx1, ly, lz = _same(vx, vy, vz)
    t = [np.empty_like(vx) for _ in range(6)]
    nx = 2 * (lx1 - 1)
    _check(lib().sc_smag(prec, _ptr(vx), _ptr(vy), _ptr(vz), *[_ptr(a, True) for a in t],
                         lx1, ly, lz, nx, ly, lz, C.c_double(delta), C.c_double(c1)))
    return t


def dynsmag(ux, uy, uz, k_test, delta, delta_test, update, cs2=0.0):
    """dynsmag.f90:1 -- returns (t, mm, lm, cs2); t = [t11 .. t33]."""
    prec, lx1, ly, lz = _same(ux, uy, uz)
    t = [np.empty_like(ux) for _ in range(6)]
    nx = 2 * (lx1 - 1)
    mm, lm, c = C.c_double(0), C.c_double(0), C.c_double(cs2)
    _check(lib().sc_dynsmag(prec, _ptr(ux), _ptr(uy), _ptr(uz), *[_ptr(a, True) for a in t],
                            lx1, ly, lz, nx, ly, lz, C.c_double(k_test), C.c_double(delta),
                            C.c_double(delta_test), C.byref(mm), C.byref(lm), C.byref(c),
                            1 if update else 0))
    return t, (mm.value if update else None), (lm.value if update else None), c.value


# ---------------------------------------------------------------------------
# handle API
# ---------------------------------------------------------------------------
def ab2v_dt(betadx, umax, dto, time, twrite):
    """The variable-step solvers' step rule (spectral_dns.f90:212-217)."""
    d = C.c_double()
    _check(lib().sc_ab2v_dt(C.c_double(betadx), C.c_double(umax), C.c_double(dto), C.c_double(time),
                            C.c_double(twrite), C.byref(d)))
    return d.value


def fp64_peak_probe():
    """FP64 FMA rate of the current GPU in TFLOP/s (sc_fp64_peak_probe: a
    bounded throughput kernel, the compute ceiling of the FP64 roofline)."""
    t = C.c_double(0)
    _check(lib().sc_fp64_peak_probe(C.byref(t)))
    return t.value


def default_params(n, precision=SC_FP32, **kw):
    p = Params()
    _check(lib().sc_default_params(C.byref(p), n, precision))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise TypeError("unknown parameter %s" % k)
        setattr(p, k, v)
    return p


class SpectralNS:
    """One solver instance (device-resident state) -- sc_create / sc_destroy."""

    def __init__(self, params: Params):
        self.p = params
        self.h = C.c_void_p()
        _check(lib().sc_create(C.byref(params), C.byref(self.h)))
        self.dtype = np.complex64 if params.precision == SC_FP32 else np.complex128
        self.shape = (params.nz, params.ny, params.nx // 2 + 1)

    def close(self):
        if self.h:
            _check(lib().sc_destroy(self.h))
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def empty(self):
        return np.zeros(self.shape, dtype=self.dtype)

    def _arrs(self, arrs):
        out = []
        for a in arrs:
            a = np.ascontiguousarray(a, dtype=self.dtype)
            if a.shape != self.shape:
                raise TypeError("expected shape %s, got %s" % (self.shape, a.shape))
            out.append(a)
        return out

    def set_state(self, vx, vy, vz):
        vx, vy, vz = self._arrs((vx, vy, vz))
        _check(lib().sc_set_state(self.h, _ptr(vx), _ptr(vy), _ptr(vz)))

    def get_state(self):
        v = [self.empty() for _ in range(3)]
        _check(lib().sc_get_state(self.h, *[_ptr(a, True) for a in v]))
        return tuple(v)

    def set_state_device(self, px, py, pz):
        _check(lib().sc_set_state_device(self.h, C.c_void_p(px), C.c_void_p(py), C.c_void_p(pz)))

    def get_state_device(self, px, py, pz):
        _check(lib().sc_get_state_device(self.h, C.c_void_p(px), C.c_void_p(py), C.c_void_p(pz)))

    def init_field(self, seed=1, kind=0, akp=4.0, u0=1.0 / np.sqrt(3.0), kmin=0.0, kmax=0.0):
        _check(lib().sc_init_field(self.h, seed, kind, C.c_double(akp), C.c_double(u0),
                                   C.c_double(kmin), C.c_double(kmax)))

    def rhs(self):
        w = [self.empty() for _ in range(3)]
        _check(lib().sc_rhs(self.h, *[_ptr(a, True) for a in w]))
        return tuple(w)

    def rk4_steps(self, n=1):
        _check(lib().sc_rk4_steps(self.h, n))

    def ab2_steps(self, n=1):
        _check(lib().sc_ab2_steps(self.h, n))

    def ab2v_pass(self, dt):
        """One pass of the variable-step IF-AB2 (spectral_dns.f90:210-290)."""
        _check(lib().sc_ab2v_pass(self.h, C.c_double(dt)))

    def ab2v_scalar_pass(self, dt, pr=1.0, scalarforced=False, meangrad=0.0, history_rhs=False):
        """One pass of spectral_dns_scalar.f90's variable-step IF-AB2 with the
        passive scalar (history_rhs: save wphi, not phi, at pass 0)."""
        _check(lib().sc_ab2v_scalar_pass(self.h, C.c_double(dt), C.c_double(pr), 1 if scalarforced else 0,
                                         C.c_double(meangrad), 1 if history_rhs else 0))

    def ab2v_state(self):
        """(pass count, previous step dto) of the variable-step IF-AB2."""
        p, d = C.c_int(), C.c_double()
        _check(lib().sc_ab2v_state(self.h, C.byref(p), C.byref(d)))
        return p.value, d.value

    def set_scalar(self, phi):
        (phi,) = self._arrs([phi])
        _check(lib().sc_set_scalar(self.h, _ptr(phi)))

    def get_scalar(self):
        phi = self.empty()
        _check(lib().sc_get_scalar(self.h, _ptr(phi, True)))
        return phi

    def rot_scalar_steps(self, n=1, om=0.0, fk1=0.0, fk2=2.5, pr=1.0, scalarforced=False, epsphi=0.0):
        """n passes of the rotating solver with its passive scalar
        (spectral_rot_dns_scalar_ft.f90:203-291)."""
        _check(lib().sc_rot_scalar_steps(self.h, n, C.c_double(om), C.c_double(fk1), C.c_double(fk2),
                                         C.c_double(pr), 1 if scalarforced else 0, C.c_double(epsphi)))

    def rot_steps(self, n=1, om=0.0, fk1=0.0, fk2=2.5):
        """n passes of the rotating solver's helical-wave IF-AB2
        (spectral_rot_dns_ft.f90:146-272) at rotation rate om, forcing band
        fk1 <= |k| < fk2 when the solver is forced."""
        _check(lib().sc_rot_steps(self.h, n, C.c_double(om), C.c_double(fk1), C.c_double(fk2)))

    def set_dt(self, dt):
        _check(lib().sc_set_dt(self.h, C.c_double(dt)))

    def set_stream(self, stream_ptr):
        _check(lib().sc_set_stream(self.h, C.c_void_p(stream_ptr)))

    def diagnostics(self):
        d = Diag()
        eks = np.zeros(self.p.nx // 2, dtype=np.float64)
        _check(lib().sc_diagnostics(self.h, C.byref(d), eks.ctypes.data_as(C.c_void_p)))
        return d.as_dict(), eks

    def adjoint(self, nsteps, checkpoint_every=20, kmin=8, kmax=16):
        """(J, grad) for J = shell enstrophy after nsteps RK4 steps; grad =
        dJ/dRe v0 + i dJ/dIm v0 in the reference layout."""
        g = [self.empty() for _ in range(3)]
        J = C.c_double(0)
        _check(lib().sc_adjoint_rk4(self.h, nsteps, checkpoint_every, kmin, kmax,
                                    *[_ptr(a, True) for a in g], C.byref(J)))
        return J.value, tuple(g)

    def output3d(self, directory, idump, file_precision=None):
        """Write the state as the reference's output3d does:
        <directory>/u{x,y,z}<idump>.dat, Fortran unformatted records."""
        fp = self.p.precision if file_precision is None else file_precision
        _check(lib().sc_output3d(self.h, str(directory).encode(), int(idump), fp))

    def input3d(self, directory, idump, file_precision=None):
        """Load the state from the reference's output3d files."""
        fp = self.p.precision if file_precision is None else file_precision
        _check(lib().sc_input3d(self.h, str(directory).encode(), int(idump), fp))

    def outputphi(self, directory, idump, file_precision=None):
        """Write the passive scalar as the reference's outputphi does:
        <directory>/phi<idump>.dat."""
        fp = self.p.precision if file_precision is None else file_precision
        _check(lib().sc_outputphi(self.h, str(directory).encode(), int(idump), fp))

    def inputphi(self, directory, idump, file_precision=None):
        """Load the passive scalar from the reference's outputphi file."""
        fp = self.p.precision if file_precision is None else file_precision
        _check(lib().sc_inputphi(self.h, str(directory).encode(), int(idump), fp))

    def set_adjoint_budget(self, nbytes):
        """Bytes for the adjoint's stage-input store (< 0: 90% of free memory,
        0: pure checkpointing with recomputation)."""
        _check(lib().sc_set_adjoint_budget(self.h, C.c_double(nbytes)))

    def adjoint_kept_segments(self):
        k = C.c_int(0)
        _check(lib().sc_adjoint_kept_segments(self.h, C.byref(k)))
        return k.value

    def adjoint_vjp(self, nsteps, lam, checkpoint_every=20):
        """(dv_T/dv_0)^T lam for the current state v_0 (left in place); lam and
        the result use the gradient convention of `adjoint`."""
        lam = self._arrs(lam)
        g = [self.empty() for _ in range(3)]
        _check(lib().sc_adjoint_rk4_vjp(self.h, nsteps, checkpoint_every, *[_ptr(a) for a in lam],
                                        *[_ptr(a, True) for a in g]))
        return tuple(g)

    def profile_enable(self, on=True):
        _check(lib().sc_profile_enable(self.h, 1 if on else 0))

    def profile_read(self, name):
        n, ms = C.c_longlong(0), C.c_double(0)
        _check(lib().sc_profile_read(self.h, name.encode(), C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def step_bytes(self):
        b = C.c_double(0)
        _check(lib().sc_step_bytes(self.h, C.byref(b)))
        return b.value


class Ensemble2D:
    """Batched 2D vorticity ensemble (sc_ens_*): members of mixed N, each a
    (N, N/2+1) complex vorticity in the reference's 2D layout."""

    def __init__(self, sizes, dts, nu8s, alpha, precision=SC_FP32):
        self.n = [int(x) for x in sizes]
        self.prec = precision
        self.dtype = np.complex64 if precision == SC_FP32 else np.complex128
        nm = len(self.n)
        a_n = (C.c_int * nm)(*self.n)
        a_dt = (C.c_double * nm)(*[float(x) for x in dts])
        a_nu = (C.c_double * nm)(*[float(x) for x in nu8s])
        self.h = C.c_void_p()
        _check(lib().sc_ens_create(precision, nm, a_n, a_dt, a_nu, C.c_double(alpha), C.byref(self.h)))

    def close(self):
        if self.h:
            _check(lib().sc_ens_destroy(self.h))
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def init(self, seeds, kpeak=6.0, energy=0.5):
        s = (C.c_int * len(seeds))(*[int(x) for x in seeds])
        _check(lib().sc_ens_init(self.h, s, C.c_double(kpeak), C.c_double(energy)))

    def set_member(self, m, w):
        w = np.ascontiguousarray(w, dtype=self.dtype)
        assert w.shape == (self.n[m], self.n[m] // 2 + 1)
        _check(lib().sc_ens_set_member(self.h, m, _ptr(w)))

    def get_member(self, m):
        w = np.zeros((self.n[m], self.n[m] // 2 + 1), dtype=self.dtype)
        _check(lib().sc_ens_get_member(self.h, m, _ptr(w, True)))
        return w

    def rk4_steps(self, nsteps, mode=0):
        _check(lib().sc_ens_rk4_steps(self.h, nsteps, mode))

    def uses_graph(self):
        return bool(lib().sc_ens_uses_graph(self.h))

    def tune(self, trial_steps=3):
        """Time every compiled launch shape on this ensemble; keep the fastest."""
        v = C.c_int(0)
        _check(lib().sc_ens_tune(self.h, trial_steps, C.byref(v)))
        return v.value

    def set_variant(self, v):
        _check(lib().sc_ens_set_variant(self.h, v))

    def variant(self):
        """(variant, {"threads", "ctas_per_sm", "tile_points", "radix", "outline"},
        ms per step of each variant in the last tuning, -1 = not timed)"""
        v, cnt = C.c_int(0), C.c_int(0)
        _check(lib().sc_ens_variant(self.h, C.byref(v), C.byref(cnt), None, None))
        ms = (C.c_double * cnt.value)()
        shape = (C.c_int * 5)()
        _check(lib().sc_ens_variant(self.h, C.byref(v), C.byref(cnt), ms, shape))
        keys = ("threads", "ctas_per_sm", "tile_points", "radix", "outline")
        return v.value, dict(zip(keys, list(shape))), list(ms)

    def set_stream(self, stream_ptr):
        _check(lib().sc_ens_set_stream(self.h, C.c_void_p(stream_ptr)))
