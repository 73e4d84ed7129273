"""FP64 CPU oracle for the pseudo-spectral Navier-Stokes step.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference leg of ``bench.py`` may import this module, and only
as the checker or as the timed CPU baseline.  The product path (the CUDA
library under ``speccodelib_gb300/``) never calls it.

What it restates
----------------
A line-by-line restatement, in NumPy/SciPy double precision, of the reference
(yili-shef/SpecCodeLib, Fortran 90 + FFTW) routines on the hot path.  Every
function cites the reference file:line it follows.

Layout
------
A spectral field is a complex128 array of shape ``(nz, ny, nx//2 + 1)`` in C
order: the same memory as the reference's Fortran array ``c(lx1, ly, lz)``
(kx fastest).  Fortran ``c(ii, jj, kk)`` is ``c[kk-1, jj-1, ii-1]`` here.  A
physical field is a float64 array of shape ``(nz, ny, nx)``.  Transforms are
unnormalised both ways exactly like FFTW's ``rfftwnd_f77_one_*``:
``c2r`` = sum_k c e^{+ik.x}; ``r2c`` = sum_x u e^{-ik.x}; callers multiply by
1/(nx ny nz) once in physical space (convec_dns.f90:15,40-42).

Parity status
-------------
The reference cannot be built here or on the GPU host (no Fortran compiler,
no FFTW; the FFTW version it links is not pinned anywhere), so this oracle is
NOT pinned to reference binaries.  It is pinned instead to a published known
answer -- the Park-Miller minimal standard generator inside ran1 reaches
z_10000 = 1043618065 from z_0 = 1 (Park and Miller, CACM 31, 1988) -- and to
the known answers the reference's own files imply
(tests/test_oracle_pins.py): the Roberts/Beltrami flow of
robertsflow.f90:23-25 (zero Lamb vector, exact e^{-2 nu t} decay under the
integrating factor), single-mode transform identities in FFTW's sign and
normalisation convention, the energy normalisation 3/2 u0^2 of
initialize.f90:362-368, the Hermitian/Nyquist rules of symmetrize.f90:32-64 and
the divergence-free output of projection.f90; for the other steppers, the
helical-basis identities of heliwave.f90 (i k x h = |k| h), exact inertial
waves of an ABC flow under the rotating solver, exact Roberts decay and
second-order convergence of the variable-step IF-AB2 on uneven steps, exact
scalar diffusion, and the forcing's injection rates (eps, epsphi).  Golden
fixtures under tests/golden/ are generated from this oracle by
tests/golden/make_golden.py.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
import subprocess
import sys

import numpy as np

try:  # scipy.fft is multi-threaded; numpy.fft is the fallback.
    import scipy.fft as _sfft

    def _irfftn(c, s, workers):
        return _sfft.irfftn(c, s=s, axes=tuple(range(c.ndim - len(s), c.ndim)),
                            norm="forward", workers=workers)

    def _rfftn(r, workers):
        return _sfft.rfftn(r, axes=tuple(range(r.ndim)), norm="backward",
                           workers=workers)
except ImportError:  # pragma: no cover
    def _irfftn(c, s, workers):
        return np.fft.irfftn(c, s=s, axes=tuple(range(c.ndim - len(s), c.ndim)),
                             norm="forward")

    def _rfftn(r, workers):
        return np.fft.rfftn(r, norm="backward")

WORKERS = int(os.environ.get("SC_ORACLE_WORKERS", "1"))

# mconstant: constant_sp.f90 makes kind sp single precision, constant.f90 and
# constant_dp.f90 make it double (the "-dp" builds).  The arithmetic here is
# FP64 throughout; MYTINY_SP is the single-precision build's tiny(1.0_sp),
# used for k2(1,1,1) in both precisions (in the double build it is
# tiny(1.0_d0): a difference confined to the mean mode).
PI_REF = 3.1415926536                          # constant_sp.f90:20, constant.f90:17 (truncated pi)
MYTINY_DP = float(np.finfo(np.float64).tiny)   # constant_sp.f90:16, constant.f90:12 tiny(1.0_dp)
MYTINY_SP = float(np.finfo(np.float32).tiny)   # constant_sp.f90:15 tiny(1.0_sp)


# --------------------------------------------------------------------------
# grid
# --------------------------------------------------------------------------
def wavenumber(nx, ny, nz):
    """kx, ky, kz (1D) and k2 (3D) -- wavenumber.f90:89-129 (low-mem 3D).

    kx = 0..nx/2; ky, kz = 0..n/2-1, -n/2..-1 (wavenumber.f90:109,115);
    k2(1,1,1) = tiny(1.0_sp) (wavenumber.f90:125).
    """
    kx = np.arange(nx // 2 + 1, dtype=np.float64)
    ky = (np.mod(np.arange(ny) + ny // 2, ny) - ny // 2).astype(np.float64)
    kz = (np.mod(np.arange(nz) + nz // 2, nz) - nz // 2).astype(np.float64)
    k2 = kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
    k2[0, 0, 0] = MYTINY_SP
    return kx, ky, kz, k2


def wavenumber2d(nx, ny):
    """2D counterpart (wavenumber.f90:187-266): k2(1,1) = tiny."""
    kx = np.arange(nx // 2 + 1, dtype=np.float64)
    ky = (np.mod(np.arange(ny) + ny // 2, ny) - ny // 2).astype(np.float64)
    k2 = ky[:, None] ** 2 + kx[None, :] ** 2
    k2[0, 0] = MYTINY_SP
    return kx, ky, k2


def c2r(c, nx, workers=None):
    """FFTW c2r, unnormalised (rfftwnd_f77_one_complex_to_real)."""
    s = c.shape[:-1] + (nx,)
    return _irfftn(c, s, WORKERS if workers is None else workers)


def r2c(r, workers=None):
    """FFTW r2c, unnormalised (rfftwnd_f77_one_real_to_complex)."""
    return _rfftn(r, WORKERS if workers is None else workers)


def packed_to_physical(c):
    """Reference packed-real view: real(c(i)) = x-point 2i-2, aimag = 2i-1
    (robertsflow.f90:33-35); the last complex column is padding."""
    nxh = c.shape[-1]
    out = np.empty(c.shape[:-1] + (2 * (nxh - 1),), dtype=np.float64)
    out[..., 0::2] = c[..., : nxh - 1].real
    out[..., 1::2] = c[..., : nxh - 1].imag
    return out


# --------------------------------------------------------------------------
# L3 operators
# --------------------------------------------------------------------------
def symmetrize3d(c):
    """symmetrize.f90:32-64 (returns a new array)."""
    c = np.array(c, dtype=np.complex128, copy=True)
    nz, ny, nxh = c.shape
    c[:, ny // 2, :] = 0.0            # :43 zero ky = -ly/2
    c[nz // 2, :, :] = 0.0            # :45 zero kz = -lz/2
    c[:, :, nxh - 1] = 0.0            # :47 zero kx = lx
    c[0, 0, 0] = 0.0                  # :49 mean mode
    # :52-57 kx = 0 plane, iz = lz/2+2..lz, all iy: c(1,iy,iz) =
    #        conj(c(1, mod(ly+1-iy,ly)+1, lz+2-iz))
    jz = np.arange(nz // 2 + 1, nz)
    jy = np.arange(ny)
    src_y = np.mod(ny - jy, ny)
    src_z = nz - jz
    c[jz[:, None], jy[None, :], 0] = np.conj(c[src_z[:, None], src_y[None, :], 0])
    # :60-62 line kx = kz = 0, iy = ly/2+2..ly
    jy2 = np.arange(ny // 2 + 1, ny)
    c[0, jy2, 0] = np.conj(c[0, ny - jy2, 0])
    return c


def hermitianize(c):
    """hermitianize.f90:1-24 (returns a new array): the kx = 0 copies of
    symmetrize.f90:52-62 alone, without its zeroing."""
    c = np.array(c, dtype=np.complex128, copy=True)
    nz, ny, nxh = c.shape
    jz = np.arange(nz // 2 + 1, nz)                                  # :10-16
    jy = np.arange(ny)
    c[jz[:, None], jy[None, :], 0] = np.conj(c[(nz - jz)[:, None], np.mod(ny - jy, ny)[None, :], 0])
    jy2 = np.arange(ny // 2 + 1, ny)                                 # :19-21
    c[0, jy2, 0] = np.conj(c[0, ny - jy2, 0])
    return c


def symmetrize2d(c):
    """symmetrize.f90:8-30 (returns a new array); c shape (ny, nxh)."""
    c = np.array(c, dtype=np.complex128, copy=True)
    ny, nxh = c.shape
    c[ny // 2, :] = 0.0
    c[:, nxh - 1] = 0.0
    c[0, 0] = 0.0
    jy = np.arange(ny // 2 + 1, ny)
    c[jy, 0] = np.conj(c[ny - jy, 0])
    return c


def dealiasing(c, k2):
    """dealiasing.f90:2-37: symmetrize, then zero k2 >= ly^2/9 (:35)."""
    ny = c.shape[1]
    c = symmetrize3d(c)
    c[k2 >= (ny * ny) / 9.0] = 0.0
    return c


def projection(vx, vy, vz, kx, ky, kz):
    """projection.f90:2-31: v <- v - k (k.v)/(k^2 + tiny)."""
    KX = kx[None, None, :]
    KY = ky[None, :, None]
    KZ = kz[:, None, None]
    tmp = KX * vx + KY * vy + KZ * vz
    tmp = tmp / (KX * KX + KY * KY + KZ * KZ + MYTINY_DP)
    return vx - KX * tmp, vy - KY * tmp, vz - KZ * tmp


def forcing_energy(vx, vy, vz, k2, fkmax):
    """K_f of force.f90:16-22: sum over k2 < fkmax^2 of |v|^2, x1/2 at kx=0."""
    tmp = np.where(k2 < fkmax * fkmax,
                   (vx * np.conj(vx) + vy * np.conj(vy) + vz * np.conj(vz)).real,
                   0.0)
    tmp[:, :, 0] *= 0.5
    return float(np.sum(tmp))


def force(wx, wy, wz, vx, vy, vz, k2, fkmax, eps):
    """force.f90:3-31: w += eps/(2 K_f) v on k2 < fkmax^2."""
    kinet = forcing_energy(vx, vy, vz, k2, fkmax)
    a = eps / (2.0 * kinet)
    m = k2 < fkmax * fkmax
    return (np.where(m, wx + a * vx, wx), np.where(m, wy + a * vy, wy),
            np.where(m, wz + a * vz, wz))


def force_rot(wx, wy, wz, vx, vy, vz, k2, fk12, fk22, eps, tiny):
    """force_rot.f90:3-29: w += a v on fk12 <= k2 < fk22 (squared bounds),
    a = eps / (2 kinet + tiny), kinet the 1/2-weighted band energy; tiny is
    the build's mytiny (constant.f90:11 / constant_sp.f90:14)."""
    m = (k2 < fk22) & (k2 >= fk12)
    tmp = np.where(m, (vx * np.conj(vx) + vy * np.conj(vy) + vz * np.conj(vz)).real, 0.0)
    tmp[:, :, 0] *= 0.5
    a = eps / (2.0 * float(np.sum(tmp)) + tiny)
    return (np.where(m, wx + a * vx, wx), np.where(m, wy + a * vy, wy),
            np.where(m, wz + a * vz, wz))


def convecphi_dns(vx, vy, vz, phi, nx):
    """convecphi_dns.f90:1-49: wphi = i k . (u phi)^, times 1/(nx ny nz)
    after the transforms (:47)."""
    ny, nz = vx.shape[1], vx.shape[0]
    const = 1.0 / float(nx * ny * nz)
    kx, ky, kz, _ = wavenumber(nx, ny, nz)
    p = c2r(phi, nx)
    fx, fy, fz = (r2c(c2r(a, nx) * p) for a in (vx, vy, vz))
    w = 1j * kx[None, None, :] * fx + 1j * ky[None, :, None] * fy + 1j * kz[:, None, None] * fz
    return w * const


def skewness(ux, nx):
    """skewness.f90:1-48: <d^3> / <d^2>^(3/2) of d = du_x/dx in physical
    space (the mean over the nx ny nz points)."""
    ny, nz = ux.shape[1], ux.shape[0]
    kx, _, _, _ = wavenumber(nx, ny, nz)
    d = c2r(1j * kx[None, None, :] * ux, nx)
    c = 1.0 / float(nx * ny * nz)
    return float(np.sum(d ** 3) * c / (np.sum(d ** 2) * c) ** 1.5)


def enstrophy_field(ux, uy, uz, nx):
    """enstrophy.f90:1-34: 1/2 |curl u|^2 at every physical point, returned
    (nz, ny, nx) (the memory of the reference's real(dp) enstr(nx,ny,nz))."""
    ny, nz = ux.shape[1], ux.shape[0]
    kx, ky, kz, _ = wavenumber(nx, ny, nz)
    w = vorticity(ux, uy, uz, kx, ky, kz)
    return 0.5 * sum(c2r(a, nx) ** 2 for a in w)


def vorticity(vx, vy, vz, kx, ky, kz):
    """w = i k x v (dns-deform.f90:265-273)."""
    KX = kx[None, None, :]
    KY = ky[None, :, None]
    KZ = kz[:, None, None]
    wx = 1j * KY * vz - 1j * KZ * vy
    wy = 1j * KZ * vx - 1j * KX * vz
    wz = 1j * KX * vy - 1j * KY * vx
    return wx, wy, wz


def convec_dns(vx, vy, vz, wx, wy, wz, nx):
    """convec_dns.f90:1-55: Lamb vector u x w, spectral in and out."""
    ny, nz = vx.shape[1], vx.shape[0]
    const = 1.0 / float(nx * ny * nz)
    ux, uy, uz = (c2r(a, nx) for a in (vx, vy, vz))
    ox, oy, oz = (c2r(a, nx) for a in (wx, wy, wz))
    lx = uy * oz - uz * oy      # :30-32
    ly = uz * ox - ux * oz      # :33-35
    lz = ux * oy - uy * ox      # :36-38
    return r2c(lx * const), r2c(ly * const), r2c(lz * const)


# --------------------------------------------------------------------------
# SGS models
# --------------------------------------------------------------------------
def strain_spectral(vx, vy, vz, kx, ky, kz):
    """S_ij in spectral space, order (11, 12, 13, 22, 23, 33) (smag.f90:21-32)."""
    KX = kx[None, None, :]
    KY = ky[None, :, None]
    KZ = kz[:, None, None]
    t11 = 1j * KX * vx
    t22 = 1j * KY * vy
    t33 = 1j * KZ * vz
    t12 = 1j * (KX * vy + KY * vx) * 0.5
    t13 = 1j * (KX * vz + KZ * vx) * 0.5
    t23 = 1j * (KY * vz + KZ * vy) * 0.5
    return [t11, t12, t13, t22, t23, t33]


def _smag_abs(s):
    """|S| = sqrt(2 S_ij S_ij) on physical fields (11,12,13,22,23,33)."""
    s11, s12, s13, s22, s23, s33 = s
    return np.sqrt(2.0 * (s11 * s11 + s22 * s22 + s33 * s33
                          + 2.0 * (s12 * s12 + s13 * s13 + s23 * s23)))


def smag(vx, vy, vz, kx, ky, kz, nx, delta, c1=0.026):
    """smag.f90:1-78: tau_ij = -2 c1 delta^2 |S| S_ij (spectral).

    c1 is hard-coded to 0.026 in the reference (smag.f90:7); here it is an
    argument with that default.
    """
    ny, nz = vx.shape[1], vx.shape[0]
    const = 1.0 / float(nx * ny * nz)
    s = [c2r(t, nx) for t in strain_spectral(vx, vy, vz, kx, ky, kz)]
    sa = _smag_abs(s)
    return [r2c(-2.0 * c1 * delta * delta * (sa * t) * const) for t in s]


def test_filter(k2, k_test):
    """Sharp spectral test filter g_test = [k2 <= k_test^2]
    (spectral_les.f90:105-109)."""
    return np.where(k2 <= k_test * k_test, 1.0, 0.0)


def dynsmag(vx, vy, vz, kx, ky, kz, g, nx, delta, delta_test, update, cs2):
    """dynsmag.f90:1-236 (Germano-Lilly, box-averaged least squares).

    Returns (tau, mm, lm, cs2).  In the non-update branch mm, lm are None and
    the passed-in cs2 is used (dynsmag.f90:196-232).
    """
    ny, nz = vx.shape[1], vx.shape[0]
    const = 1.0 / float(nx * ny * nz)
    d2 = delta * delta
    dt2 = delta_test * delta_test
    sspec = strain_spectral(vx, vy, vz, kx, ky, kz)
    s = [c2r(t, nx) for t in sspec]
    sa = _smag_abs(s)
    if update:
        # L_ij (:28-77)
        u = [c2r(a, nx) for a in (vx, vy, vz)]
        gu = [c2r(g * a, nx) for a in (vx, vy, vz)]
        pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
        L = []
        for (i, j) in pairs:
            f = c2r(g * r2c(u[i] * u[j]) * const, nx)
            L.append(f - gu[i] * gu[j])
        # M_ij (:79-168)
        s2 = [r2c(2.0 * d2 * (sa * t) * const) for t in s]       # :110-122
        gs = [c2r(g * t, nx) for t in sspec]                        # :88-130
        gsa = _smag_abs(gs)
        tpart = [-2.0 * dt2 * (gsa * t) for t in gs]                 # :140-145
        M = [c2r(g * s2[n], nx) + tpart[n] for n in range(6)]       # :148-168
        w = [1.0, 2.0, 2.0, 1.0, 2.0, 1.0]
        mm = float(sum(w[n] * np.sum(M[n] * M[n]) for n in range(6)))   # :170-176
        lm = float(sum(w[n] * np.sum(L[n] * M[n]) for n in range(6)))   # :178-184
        cs2 = lm / mm                                                    # :186
        tau = [-cs2 * t for t in s2]                                     # :188-193
        return tau, mm, lm, cs2
    tau = [r2c(-cs2 * 2.0 * d2 * (sa * t) * const) for t in s]          # :220-232
    return tau, None, None, cs2


def sgs_divergence(tau, kx, ky, kz):
    """-i k_j tau_ij (spectral_les.f90:232-234)."""
    t11, t12, t13, t22, t23, t33 = tau
    KX = kx[None, None, :]
    KY = ky[None, :, None]
    KZ = kz[:, None, None]
    return (-1j * (KX * t11 + KY * t12 + KZ * t13),
            -1j * (KX * t12 + KY * t22 + KZ * t23),
            -1j * (KX * t13 + KY * t23 + KZ * t33))


# --------------------------------------------------------------------------
# parameters and right-hand sides
# --------------------------------------------------------------------------
@dataclasses.dataclass
class Params:
    nx: int
    ny: int = 0
    nz: int = 0
    nu: float = 0.01
    dt: float = 2e-3
    forced: bool = True
    eps: float = 0.1
    fkmax: float = 2.5
    kcut: float = 0.0          # 0 -> 2*(nx/2)/3 (dns-deform.f90:75)
    sgs: str = "none"          # "none" | "smag" | "dynsmag"
    c1: float = 0.026          # smag.f90:7
    delta: float = 0.0         # 0 -> pi/kcut (spectral_les.f90:87)
    delta_ratio: float = 2.0   # spectral_les.f90:16
    dyn_every: int = 10        # spectral_les.f90:17
    mask: str = "after_step"   # "after_step" (dns-deform.f90:233-237) | "rhs_and_step"

    def __post_init__(self):
        self.ny = self.ny or self.nx
        self.nz = self.nz or self.nx
        if self.kcut == 0.0:
            self.kcut = 2.0 * (self.nx // 2) / 3.0
        if self.delta == 0.0:
            self.delta = PI_REF / self.kcut

    @property
    def k_test(self):
        return self.kcut / self.delta_ratio          # spectral_les.f90:89

    @property
    def delta_test(self):
        return self.delta_ratio * self.delta         # spectral_les.f90:90


class Grid:
    def __init__(self, p: Params):
        self.p = p
        self.kx, self.ky, self.kz, self.k2 = wavenumber(p.nx, p.ny, p.nz)
        self.g = test_filter(self.k2, p.k_test)


def ratesdudt(v, grid: Grid, sgs_state=None, symmetrize=True):
    """Right-hand side of dns-deform.f90:259-288 (plus the optional SGS term
    of spectral_les.f90:204-234, applied before symmetrize/projection).

    v: tuple of three spectral fields.  sgs_state: dict with keys 'cs2',
    'update' for dynsmag; receives 'mm', 'lm', 'cs2' back.  symmetrize=False
    leaves out :281-283, as the variable-step solvers do.
    """
    p = grid.p
    kx, ky, kz, k2 = grid.kx, grid.ky, grid.kz, grid.k2
    vx, vy, vz = v
    wx, wy, wz = vorticity(vx, vy, vz, kx, ky, kz)                     # :265-273
    wx, wy, wz = convec_dns(vx, vy, vz, wx, wy, wz, p.nx)              # :276
    if p.forced:
        wx, wy, wz = force(wx, wy, wz, vx, vy, vz, k2, p.fkmax, p.eps)  # :279
    if p.sgs != "none":
        if p.sgs == "smag":
            tau = smag(vx, vy, vz, kx, ky, kz, p.nx, p.delta, p.c1)
        else:
            st = sgs_state if sgs_state is not None else {"cs2": 0.0, "update": True}
            tau, mm, lm, cs2 = dynsmag(vx, vy, vz, kx, ky, kz, grid.g, p.nx,
                                        p.delta, p.delta_test, st["update"], st["cs2"])
            st["cs2"] = cs2
            if mm is not None:
                st["mm"], st["lm"] = mm, lm
        dx, dy, dz = sgs_divergence(tau, kx, ky, kz)
        wx, wy, wz = wx + dx, wy + dy, wz + dz
    if symmetrize:
        wx, wy, wz = symmetrize3d(wx), symmetrize3d(wy), symmetrize3d(wz)  # :281-283
    wx, wy, wz = projection(wx, wy, wz, kx, ky, kz)                    # :286
    if p.mask == "rhs_and_step":
        m = k2 >= p.kcut * p.kcut
        wx, wy, wz = (np.where(m, 0.0, a) for a in (wx, wy, wz))
    return wx, wy, wz


def mask_state(v, grid: Grid):
    """2/3 truncation of the state after the step (dns-deform.f90:233-237)."""
    m = grid.k2 >= grid.p.kcut * grid.p.kcut
    return tuple(np.where(m, 0.0, a) for a in v)


def rk4_step(v, grid: Grid, sgs_state=None, dyn_update=None):
    """One integrating-factor RK4 step, literally dns-deform.f90:160-237.

    k2e = exp(-nu k2 dt/2) (dns-deform.f90:90).  For dynsmag, the dynamic
    coefficient is recomputed only on the first stage when dyn_update is True.
    """
    p = grid.p
    dt = p.dt
    k2e = np.exp(-p.nu * grid.k2 * dt / 2)

    def rhs(s, first):
        if sgs_state is not None:
            sgs_state["update"] = bool(dyn_update) and first
        return ratesdudt(s, grid, sgs_state)

    vx, vy, vz = v
    w = rhs((vx, vy, vz), True)                                        # :164
    ku = [dt * a for a in w]                                           # :165-167
    du = list(ku)
    s = [k2e * (a + b / 2) for a, b in zip((vx, vy, vz), ku)]          # :177-179
    w = rhs(s, False)
    ku = [dt * a / k2e for a in w]                                     # :182-184
    du = [a + 2 * b for a, b in zip(du, ku)]
    s = [k2e * (a + b / 2) for a, b in zip((vx, vy, vz), ku)]          # :194-196
    w = rhs(s, False)
    ku = [dt * a / k2e for a in w]                                     # :199-201
    du = [a + 2 * b for a, b in zip(du, ku)]
    s = [k2e * k2e * (a + b) for a, b in zip((vx, vy, vz), ku)]        # :211-213
    w = rhs(s, False)
    ku = [dt * a / k2e / k2e for a in w]                               # :216-218
    du = [a + b for a, b in zip(du, ku)]
    vn = [k2e * k2e * (a + b / 6) for a, b in zip((vx, vy, vz), du)]   # :226-228
    return mask_state(vn, grid)


def rk4_run(v, grid: Grid, nsteps, sgs_state=None):
    """nsteps RK4 steps; dynsmag coefficient refreshed on steps that are
    multiples of dyn_every (counted from 0)."""
    for n in range(nsteps):
        v = rk4_step(v, grid, sgs_state, dyn_update=(n % grid.p.dyn_every == 0))
    return v


def ab2_rhs(v, grid: Grid):
    """RHS of the production IF-AB2 solver, specdns-forced-omp-ft.f90:180-221:
    vorticity, Lamb vector, forcing, projection with /k2 (no symmetrize)."""
    p = grid.p
    kx, ky, kz, k2 = grid.kx, grid.ky, grid.kz, grid.k2
    vx, vy, vz = v
    wx, wy, wz = vorticity(vx, vy, vz, kx, ky, kz)
    wx, wy, wz = convec_dns(vx, vy, vz, wx, wy, wz, p.nx)
    if p.forced:
        wx, wy, wz = force(wx, wy, wz, vx, vy, vz, k2, p.fkmax, p.eps)
    KX, KY, KZ = kx[None, None, :], ky[None, :, None], kz[:, None, None]
    t = (KX * wx.real + KY * wy.real + KZ * wz.real) / k2             # :211-214
    wx = wx - KX * t
    wy = wy - KY * t
    wz = wz - KZ * t
    t = (KX * wx.imag + KY * wy.imag + KZ * wz.imag) / k2             # :216-219
    wx = wx - 1j * KX * t
    wy = wy - 1j * KY * t
    wz = wz - 1j * KZ * t
    return wx, wy, wz


def ab2_run(v, grid: Grid, nhalf_steps):
    """IF-AB2 of specdns-forced-omp-ft.f90:224-287 for `nhalf_steps` passes of
    its loop (pass 0 = Euler half step, pass 1 = midpoint restart from the
    initial field, then AB2).  Returns (v, time)."""
    p = grid.p
    dt = p.dt
    dt_h = 0.5 * dt
    expk2 = np.exp(-grid.k2 * p.nu * dt)                             # :92
    expk2[0, 0, 0] = 1.0                                             # :93
    sq = np.sqrt(expk2)
    o = list(v)
    o0 = None
    v = list(v)
    t = 0.0
    for istep in range(nhalf_steps):
        w = ab2_rhs(v, grid)
        if istep == 0:                                               # :225-234
            v = [(a + dt_h * b) * sq for a, b in zip(v, w)]
            t += dt_h
            o0 = w
        elif istep == 1:                                             # :236-251
            v = [a * expk2 + dt * b * sq for a, b in zip(o, w)]
            t += dt_h
            o = o0
        else:                                                        # :255-270
            v = [(a + (3.0 * b - expk2 * c) * dt_h) * expk2 for a, b, c in zip(v, w, o)]
            o = w
            t += dt
        v = [a.copy() for a in v]
        for a in v:
            a[0, 0, 0] = 0.0                                         # :277-279
        m = grid.k2 >= (2.0 * (p.nx // 2) / 3.0) ** 2
        v = [np.where(m, 0.0, a) for a in v]                         # :283-287
    return tuple(v), t


# --------------------------------------------------------------------------
# variable-step IF-AB2 (spectral_dns.f90, spectral_les.f90)
# --------------------------------------------------------------------------
def ab2v_rhs(v, grid: Grid, sgs_state=None):
    """Right-hand side of the variable-step solvers: spectral_dns.f90:173-208
    (vorticity, Lamb vector, forcing :189-205, projection :208) and, with an
    SGS model, spectral_les.f90:199-238 (dynsmag :205-207, forcing :214-230,
    SGS divergence :232-234, projection :237-238): ratesdudt without
    symmetrize."""
    return ratesdudt(v, grid, sgs_state, symmetrize=False)


def ab2v_dt(betadx, umax, dto, time, twrite):
    """Step of spectral_dns.f90:212-217 (spectral_les.f90:242-247): the CFL
    step betadx / umax, at most 3 dto, shortened to land on the next output
    time twrite (halved when it would leave a sliver under 0.2 dt)."""
    dt = min(betadx / umax, 3.0 * dto)
    if dt >= twrite - time:
        dt = twrite - time
    elif twrite - time - dt < 0.2 * dt:
        dt = 0.5 * (twrite - time)
    return dt


def ab2v_weights(ipass, dt, dto):
    """(S, ek, delta) of spectral_dns.f90:231-235 (pass 1) and :253-257
    (passes >= 2); pass 0 has none."""
    dtt = dt / dto
    if ipass == 1:
        return 0.5 * (1.0 + dtt * dtt), 0.5 * (1.0 - dtt * dtt), 0.5 * dto * (1.0 + dtt) ** 2
    return (1.0 + 0.5 * dtt) * dt, -0.5 * dtt * dt, 0.0


def ab2v_scalar_run(v, phi, grid: Grid, dts, pr, scalarforced=False, meangrad=0.0, history="as_written",
                    trace=None):
    """Passes of spectral_dns_scalar.f90:222-342, the variable-step IF-AB2
    with a passive scalar.  Its `symmetrize(w, k2, lx1, ly, lz)` calls
    (:248-251) have five arguments, matching none of symmetrize.f90's forms;
    dealiasing.f90:1 states that dealiasing differs from symmetrize only in
    its last statement (the 2/3 mask), so they are read as symmetrize3d with
    an unused k2.  Per pass: the velocity RHS of ratesdudt (vorticity, Lamb
    vector, force, symmetrize, projection, :222-254); wphi = convecphi_dns
    (:236), minus meangrad v_z when scalarforced (:244-246; the reference
    derives meangrad from epsphi, u0, phirms and a placeholder constant,
    :8, :87), symmetrized (:251); then the variable-step updates of
    spectral_dns.f90 for v and, with exp(-nu k2 dt / pr), for phi
    (:265-339), with no truncation of v afterwards.  As written, pass 0
    saves phi after its update as the scalar's history (outputphi(phi, 0),
    :278, read back at :308), not wphi: pass 2 uses that value; the
    velocity's history is w (:277).  history="rhs" saves wphi instead (the
    evident intent, as spectral_rot_dns_scalar_ft.f90:237 does).  Returns
    (v, phi, time, dto); with a list
    `trace`, each pass appends (w, wphi, v after it, phi after it)."""
    p = grid.p
    k2 = grid.k2
    v0 = [np.array(a, dtype=np.complex128) for a in v]
    v = list(v0)
    phi0 = np.array(phi, dtype=np.complex128)
    phi = phi0
    o = o0 = ophi = None
    t, dto = 0.0, None
    for ip, dt in enumerate(dts):
        w = ratesdudt(v, grid)
        wphi = convecphi_dns(v[0], v[1], v[2], phi, p.nx)
        if scalarforced:
            wphi = wphi - meangrad * v[2]
        wphi = symmetrize3d(wphi)
        e1, e1p = np.exp(-p.nu * k2 * dt), np.exp(-p.nu * k2 * dt / pr)
        if ip == 0:
            v = [(a + dt * b) * e1 for a, b in zip(v, w)]
            phi = (phi + dt * wphi) * e1p
            dto = dt
            o0, ophi = w, (phi if history == "as_written" else wphi)   # :277-278
        elif ip == 1:
            S, ek, dl = ab2v_weights(1, dt, dto)
            e0, e0p = np.exp(-p.nu * k2 * dto), np.exp(-p.nu * k2 * dto / pr)
            v = [(S * a0 * e0 + ek * a + dl * b) * e1 for a0, a, b in zip(v0, v, w)]
            phi = (S * phi0 * e0p + ek * phi + dl * wphi) * e1p
            dto = dt + dto
            o = o0                                                     # :307-308
        else:
            S, ek, _ = ab2v_weights(ip, dt, dto)
            e0, e0p = np.exp(-p.nu * k2 * dto), np.exp(-p.nu * k2 * dto / pr)
            v = [(a + S * b + ek * c * e0) * e1 for a, b, c in zip(v, w, o)]
            phi = (phi + S * wphi + ek * ophi * e0p) * e1p
            o, ophi = w, wphi
            dto = dt
        t += dt
        if trace is not None:
            trace.append((w, wphi, tuple(v), phi))
    return tuple(v), phi, t, dto


def ab2v_run(v, grid: Grid, dts, sgs_state=None, trace=None):
    """Passes of the variable-step IF-AB2 of spectral_dns.f90:210-290
    (spectral_les.f90:240-316) with steps dts[p]: pass 0 an integrating-factor
    Euler step (:220-228), pass 1 a restart from the initial field over
    dt0 + dt1 weighted by dt1/dt0 (:230-250), later passes AB2 weighted by
    dt/dto with the previous right-hand side (:252-275); after each pass
    v = 0 at k2 >= kcut^2 and at the mean mode (:281-290; spectral_dns.f90
    cuts at lx^2, spectral_les.f90 at kcut^2: the grid's kcut).  With a
    dynsmag grid the coefficient is refreshed on passes 0, 1, 11, 21, ...
    (update is .true. at first and then mod(istep, 10) == 0 of the previous
    pass, spectral_les.f90:140,205-208).  Returns (v, time, dto); with a list
    `trace`, each pass appends (its right-hand side, v after it)."""
    p = grid.p
    k2 = grid.k2
    v0 = [np.array(a, dtype=np.complex128) for a in v]             # :103-105
    v = list(v0)
    o = o0 = None
    t, dto = 0.0, None
    if p.sgs == "dynsmag" and sgs_state is None:
        sgs_state = {"cs2": 0.0, "update": True}
    for ip, dt in enumerate(dts):
        if p.sgs == "dynsmag":
            sgs_state["update"] = ip == 0 or (ip - 1) % p.dyn_every == 0
        w = ab2v_rhs(v, grid, sgs_state)
        e1 = np.exp(-p.nu * k2 * dt)
        if ip == 0:
            v = [(a + dt * b) * e1 for a, b in zip(v, w)]
            dto = dt
            o0 = w                                                     # :228 (written out)
        elif ip == 1:
            S, ek, dl = ab2v_weights(1, dt, dto)
            e0 = np.exp(-p.nu * k2 * dto)
            v = [(S * a0 * e0 + ek * a + dl * b) * e1 for a0, a, b in zip(v0, v, w)]
            dto = dt + dto
            o = o0                                                     # :250 (read back)
        else:
            S, ek, _ = ab2v_weights(ip, dt, dto)
            e0 = np.exp(-p.nu * k2 * dto)
            v = [(a + S * b + ek * c * e0) * e1 for a, b, c in zip(v, w, o)]
            o = w
            dto = dt
        t += dt
        m = k2 >= p.kcut * p.kcut
        v = [np.where(m, 0.0, a) for a in v]
        for a in v:
            a[0, 0, 0] = 0.0
        if trace is not None:
            trace.append((w, tuple(v)))
    return tuple(v), t, dto


# --------------------------------------------------------------------------
# rotating solver: helical-wave IF-AB2 (spectral_rot_dns_ft.f90)
# --------------------------------------------------------------------------
def heliwave(kx, ky, kz, k2):
    """Positive-helicity unit vectors h+ at every mode, heliwave.f90:57-96
    (the low-memory form the rotating solver calls with 1D kx, ky, kz;
    spectral_rot_dns_ft.f90:24,114).  h- = conj(h+), i k x h+ = |k| h+.

    Rows with ky = kz = 0 (:73-81) use k2d = max(sqrt(kx^2 + ky^2),
    smallest); the others (:82-91) k2d = sqrt(kz^2 + ky^2).  The floor only
    acts at the mean mode, whose numerators are all zero, so h = 0 there."""
    s = np.sqrt(2.0) / 2.0
    KX = np.broadcast_to(kx[None, None, :], k2.shape)
    KY = np.broadcast_to(ky[None, :, None], k2.shape)
    KZ = np.broadcast_to(kz[:, None, None], k2.shape)
    k = np.sqrt(k2)
    with np.errstate(divide="ignore", invalid="ignore"):
        k2d = np.sqrt(KZ * KZ + KY * KY)
        hx = s * (1j * (KY * KY + KZ * KZ) / k / k2d)
        hy = s * (-KZ / k2d - 1j * KX * KY / k / k2d)
        hz = s * (KY / k2d - 1j * KZ * KX / k / k2d)
    smallest = 2.0 * float(np.finfo(np.float32).eps)      # constant_sp.f90:7
    kxa, k0 = kx, k[0, 0, :]
    k2d0 = np.maximum(np.abs(kxa), smallest)               # ky = 0 on this row
    hx[0, 0, :] = s * (-0.0 / k2d0 - 1j * kxa * 0.0 / k0 / k2d0)
    hy[0, 0, :] = s * (kxa / k2d0 - 1j * 0.0 * 0.0 / k0 / k2d0)
    hz[0, 0, :] = s * (1j * (kxa * kxa) / k0 / k2d0)
    return hx, hy, hz


def rot_factors(grid: Grid, om):
    """efp = exp(-k2 nu dt + 2 i dt kz om / (sqrt(k2) + tiny)) and efm with
    the opposite phase (spectral_rot_dns_ft.f90:101-111); sqrt is the
    principal complex square root, as Fortran's."""
    p = grid.p
    KZ = grid.kz[:, None, None]
    ph = 2.0 * p.dt * KZ * om / (np.sqrt(grid.k2) + MYTINY_SP)
    efp = np.exp(-grid.k2 * p.nu * p.dt + 1j * ph)
    efm = np.exp(-grid.k2 * p.nu * p.dt - 1j * ph)
    return efp, efm, np.sqrt(efp), np.sqrt(efm)


def rot_rhs(v, grid: Grid, fk1, fk2):
    """Right-hand side of the rotating solver, spectral_rot_dns_ft.f90:189-211:
    vorticity (:190-198), Lamb vector (:201), force_rot on the band
    fk1^2 <= k2 < fk2^2 when forced (:204), symmetrize of each component
    (:206-208), projection with +tiny (:211)."""
    p = grid.p
    kx, ky, kz, k2 = grid.kx, grid.ky, grid.kz, grid.k2
    vx, vy, vz = v
    wx, wy, wz = vorticity(vx, vy, vz, kx, ky, kz)
    wx, wy, wz = convec_dns(vx, vy, vz, wx, wy, wz, p.nx)
    if p.forced:
        wx, wy, wz = force_rot(wx, wy, wz, vx, vy, vz, k2, fk1 * fk1, fk2 * fk2, p.eps, MYTINY_SP)
    wx, wy, wz = symmetrize3d(wx), symmetrize3d(wy), symmetrize3d(wz)
    return projection(wx, wy, wz, kx, ky, kz)


def rot_run(v, grid: Grid, npasses, om, fk1=0.0, fk2=2.5, trace=None):
    """`npasses` passes of the rotating solver's loop,
    spectral_rot_dns_ft.f90:146-272: the state is the pair of helical
    amplitudes a+ = v . conj(h), a- = v . h (:132-133); pass 0 is an Euler
    half step (:215-223), pass 1 a midpoint restart from the initial field
    (:225-237), then AB2 with the previous right-hand side (:239-256); after
    each pass v = a+ h + a- conj(h) with the 2/3 truncation (:261-270), the
    amplitudes themselves are not truncated.  Returns (v, (a+, a-), time).
    With a list `trace`, each pass appends (its right-hand side, v after it)."""
    p = grid.p
    dt = p.dt
    dt_h = 0.5 * dt                                                  # :135
    hx, hy, hz = heliwave(grid.kx, grid.ky, grid.kz, grid.k2)
    efp, efm, sqp, sqm = rot_factors(grid, om)
    kcut2 = (2.0 * (p.nx // 2) / 3.0) ** 2                           # :85-86
    v = [np.array(a, dtype=np.complex128) for a in v]
    ox, oy, oz = v                                                   # :129-131
    ap = v[0] * np.conj(hx) + v[1] * np.conj(hy) + v[2] * np.conj(hz)
    am = v[0] * hx + v[1] * hy + v[2] * hz
    o0 = None
    t = 0.0
    for istep in range(npasses):
        wx, wy, wz = rot_rhs(v, grid, fk1, fk2)
        if istep == 0:
            ap = (ap + dt_h * (wx * np.conj(hx) + wy * np.conj(hy) + wz * np.conj(hz))) * sqp
            am = (am + dt_h * (wx * hx + wy * hy + wz * hz)) * sqm
            t += dt_h
            o0 = (wx, wy, wz)                                        # :223 (written out)
        elif istep == 1:
            ap = ((ox * np.conj(hx) + oy * np.conj(hy) + oz * np.conj(hz)) * efp
                  + dt * (wx * np.conj(hx) + wy * np.conj(hy) + wz * np.conj(hz)) * sqp)
            am = (ox * hx + oy * hy + oz * hz) * efm + dt * (wx * hx + wy * hy + wz * hz) * sqm
            t += dt_h
            ox, oy, oz = o0                                          # :235 (read back)
        else:
            tx, ty, tz = 3.0 * wx - efp * ox, 3.0 * wy - efp * oy, 3.0 * wz - efp * oz
            ap = (ap + dt_h * (tx * np.conj(hx) + ty * np.conj(hy) + tz * np.conj(hz))) * efp
            tx, ty, tz = 3.0 * wx - efm * ox, 3.0 * wy - efm * oy, 3.0 * wz - efm * oz
            am = (am + dt_h * (tx * hx + ty * hy + tz * hz)) * efm
            ox, oy, oz = wx, wy, wz
            t += dt
        v = [ap * hx + am * np.conj(hx), ap * hy + am * np.conj(hy), ap * hz + am * np.conj(hz)]
        m = grid.k2 >= kcut2
        v = [np.where(m, 0.0, a) for a in v]
        if trace is not None:
            trace.append(((wx, wy, wz), tuple(v)))
    return tuple(v), (ap, am), t


def forcephi(phi, wphi, k2, fkmax, epsphi):
    """forcephi.f90:1-27: wphi += a phi on k2 < fkmax^2, a = epsphi / (2
    kinet), kinet the 1/2-weighted variance of phi there."""
    m = k2 < fkmax * fkmax
    tmp = np.where(m, (phi * np.conj(phi)).real, 0.0)
    tmp[:, :, 0] *= 0.5
    a = epsphi / (2.0 * float(np.sum(tmp)))
    return np.where(m, wphi + a * phi, wphi)


def forcephi_rot(phi, wphi, k2, fk1, fk2, epsphi):
    """forcephi_rot.f90:1-27: wphi += a phi on fk1^2 <= k2 < fk2^2,
    a = epsphi / (2 kinet), kinet the 1/2-weighted band variance of phi."""
    m = (k2 < fk2 * fk2) & (k2 >= fk1 * fk1)
    tmp = np.where(m, (phi * np.conj(phi)).real, 0.0)
    tmp[:, :, 0] *= 0.5
    a = epsphi / (2.0 * float(np.sum(tmp)))
    return np.where(m, wphi + a * phi, wphi)


def rot_scalar_run(v, phi, grid: Grid, npasses, om, fk1, fk2, pr, scalarforced=False, epsphi=0.0,
                   trace=None):
    """`npasses` passes of the rotating solver with a passive scalar,
    spectral_rot_dns_scalar_ft.f90:203-291 (the program as written does not
    compile: :20 declares kx, ky, kz rank 3 and :84 allocates them rank 1;
    this follows its evident intent with the 1D wavenumbers of
    spectral_rot_dns_ft.f90).  Per pass: Lamb vector and wphi =
    convecphi_dns (:209-210); force_rot with fk1, fk2 passed as its squared
    bounds, so the band is fk1 <= k2 < fk2 (:213); forcephi_rot on
    fk1^2 <= k2 < fk2^2 (:214); dealiasing (symmetrize, then zero
    k2 >= ly^2/9) of w and wphi (:216-219); projection (:222); the helical
    AB2 of rot_run for the velocity and the same schedule for phi with
    efphi = exp(-nu k2 dt / pr) (:104, :230, :249, :278-279); the rebuilt
    velocity is not truncated (:289-291).  Returns (v, phi, (a+, a-), time);
    with a list `trace`, each pass appends (w, wphi, v after it, phi after it)."""
    p = grid.p
    dt = p.dt
    dt_h = 0.5 * dt
    kx, ky, kz, k2 = grid.kx, grid.ky, grid.kz, grid.k2
    hx, hy, hz = heliwave(kx, ky, kz, k2)
    efp, efm, sqp, sqm = rot_factors(grid, om)
    efphi = np.exp(-k2 * p.nu * dt / pr)
    sqphi = np.sqrt(efphi)
    v = [np.array(a, dtype=np.complex128) for a in v]
    phi = np.array(phi, dtype=np.complex128)
    ox, oy, oz = v                                                   # :133-135
    ophi = phi                                                       # :136
    ap = v[0] * np.conj(hx) + v[1] * np.conj(hy) + v[2] * np.conj(hz)
    am = v[0] * hx + v[1] * hy + v[2] * hz
    o0 = ophi0 = None
    t = 0.0
    for istep in range(npasses):
        vx, vy, vz = v
        wx, wy, wz = vorticity(vx, vy, vz, kx, ky, kz)
        wx, wy, wz = convec_dns(vx, vy, vz, wx, wy, wz, p.nx)
        wphi = convecphi_dns(vx, vy, vz, phi, p.nx)
        if p.forced:
            wx, wy, wz = force_rot(wx, wy, wz, vx, vy, vz, k2, fk1, fk2, p.eps, MYTINY_SP)
        if scalarforced:
            wphi = forcephi_rot(phi, wphi, k2, fk1, fk2, epsphi)
        wx, wy, wz, wphi = (dealiasing(a, k2) for a in (wx, wy, wz, wphi))
        wx, wy, wz = projection(wx, wy, wz, kx, ky, kz)
        if istep == 0:
            ap = (ap + dt_h * (wx * np.conj(hx) + wy * np.conj(hy) + wz * np.conj(hz))) * sqp
            am = (am + dt_h * (wx * hx + wy * hy + wz * hz)) * sqm
            phi = (phi + dt_h * wphi) * sqphi
            t += dt_h
            o0, ophi0 = (wx, wy, wz), wphi                           # :236-237 (written out)
        elif istep == 1:
            ap = ((ox * np.conj(hx) + oy * np.conj(hy) + oz * np.conj(hz)) * efp
                  + dt * (wx * np.conj(hx) + wy * np.conj(hy) + wz * np.conj(hz)) * sqp)
            am = (ox * hx + oy * hy + oz * hz) * efm + dt * (wx * hx + wy * hy + wz * hz) * sqm
            phi = ophi * efphi + dt * wphi * sqphi
            t += dt_h
            (ox, oy, oz), ophi = o0, ophi0                           # :255-256 (read back)
        else:
            tx, ty, tz = 3.0 * wx - efp * ox, 3.0 * wy - efp * oy, 3.0 * wz - efp * oz
            ap = (ap + dt_h * (tx * np.conj(hx) + ty * np.conj(hy) + tz * np.conj(hz))) * efp
            tx, ty, tz = 3.0 * wx - efm * ox, 3.0 * wy - efm * oy, 3.0 * wz - efm * oz
            am = (am + dt_h * (tx * hx + ty * hy + tz * hz)) * efm
            ox, oy, oz = wx, wy, wz
            phi = (phi + dt_h * (3.0 * wphi - ophi * efphi)) * efphi
            ophi = wphi
            t += dt
        v = [ap * hx + am * np.conj(hx), ap * hy + am * np.conj(hy), ap * hz + am * np.conj(hz)]
        if trace is not None:
            trace.append(((wx, wy, wz), wphi, tuple(v), phi))
    return tuple(v), phi, (ap, am), t


# --------------------------------------------------------------------------
# diagnostics (FP64)
# --------------------------------------------------------------------------
def _q(v):
    q = sum((a * np.conj(a)).real for a in v)
    q[:, :, 0] *= 0.5
    return q


def energy(v):
    """E = sum of 1/2-weighted |v|^2 (specdns-forced-omp-ft.f90:142-144)."""
    return float(np.sum(_q(v)))


def spectrum(v, k2, nx):
    """Shell spectrum, ll = floor(sqrt(k2)+.5), 1 <= ll <= lx
    (specdns-forced-omp-ft.f90:159-176).  Returns array eks[0..lx-1]."""
    lx = nx // 2
    q = _q(v)
    ll = np.floor(np.sqrt(k2) + 0.5).astype(np.int64)
    m = (ll >= 1) & (ll <= lx)
    return np.bincount(ll[m] - 1, weights=q[m], minlength=lx)[:lx]


def dissipation(v, k2, nu):
    """eps = 2 nu sum k^2 q(k) over modes (the per-mode form of
    meaneps.f90:37-44)."""
    kk = k2.copy()
    kk[0, 0, 0] = 0.0
    return float(2.0 * nu * np.sum(kk * _q(v)))


def enstrophy(v, k2):
    kk = k2.copy()
    kk[0, 0, 0] = 0.0
    return float(np.sum(kk * _q(v)))


def max_divergence(v, kx, ky, kz):
    """max |k . v| over all modes."""
    vx, vy, vz = v
    d = kx[None, None, :] * vx + ky[None, :, None] * vy + kz[:, None, None] * vz
    return float(np.max(np.abs(d)))


def max_velocity(v, nx):
    """max over grid points of |u| (CFL diagnostic)."""
    u = [c2r(a, nx) for a in v]
    return float(np.sqrt(np.max(u[0] ** 2 + u[1] ** 2 + u[2] ** 2)))


# --------------------------------------------------------------------------
# seeded initial fields (initialize.f90)
# --------------------------------------------------------------------------
_LIB = None


def _ran1_lib():
    """Compile oracle/ran1.c on first use (gcc), or load the prebuilt copy."""
    global _LIB
    if _LIB is not None:
        return _LIB
    here = os.path.dirname(os.path.abspath(__file__))
    so = os.path.join(here, "_build", "liboracle_ran1.so")
    src = os.path.join(here, "ran1.c")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        build_c(here)
    lib = ctypes.CDLL(so)
    lib.oracle_gauss_fields.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int32,
                                        ctypes.c_void_p]
    lib.oracle_ran1_sequence.argtypes = [ctypes.c_int32, ctypes.c_int64,
                                         ctypes.c_void_p]
    lib.oracle_ran1_state_after.argtypes = [ctypes.c_int32, ctypes.c_int64]
    lib.oracle_ran1_state_after.restype = ctypes.c_int32
    lib.oracle_park_miller_after.argtypes = [ctypes.c_int32, ctypes.c_int64]
    lib.oracle_park_miller_after.restype = ctypes.c_int32
    _LIB = lib
    return lib


def build_c(here=None):
    """Compile the oracle's C helper into oracle/_build/."""
    here = here or os.path.dirname(os.path.abspath(__file__))
    os.makedirs(os.path.join(here, "_build"), exist_ok=True)
    so = os.path.join(here, "_build", "liboracle_ran1.so")
    tmp = so + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-o", tmp,
                           os.path.join(here, "ran1.c"), "-lm"])
    os.replace(tmp, so)
    return so


def ran1_state_after(seed, ncalls):
    """ran1's integer state idum after `ncalls` calls (initialize.f90:516-548)."""
    return int(_ran1_lib().oracle_ran1_state_after(seed, ncalls))


def park_miller_after(z0, n):
    """z_n of the Park-Miller minimal standard generator (the multiplier 16807,
    modulus 2^31 - 1 and Schrage constants of initialize.f90:521-523)."""
    return int(_ran1_lib().oracle_park_miller_after(z0, n))


def ran1_sequence(seed, count):
    out = np.empty(count, dtype=np.float64)
    _ran1_lib().oracle_ran1_sequence(seed, count, out.ctypes.data)
    return out


def ran1_sequence_py(seed, count):
    """Pure-Python NR ran1 (initialize.f90:516-548), for cross-checking the C
    helper on short sequences."""
    ia, im, iq, ir, ntab = 16807, 2147483647, 127773, 2836, 32
    ndiv = 1 + (im - 1) // ntab
    am = 1.0 / im
    rnmx = 1.0 - 1.2e-7
    iv = [0] * ntab
    idum = max(-seed, 1)                       # initialize.f90:530
    for j in range(ntab + 8, 0, -1):
        k = idum // iq
        idum = ia * (idum - k * iq) - ir * k
        if idum < 0:
            idum += im
        if j <= ntab:
            iv[j - 1] = idum
    iy = iv[0]
    out = []
    for _ in range(count):
        k = idum // iq
        idum = ia * (idum - k * iq) - ir * k
        if idum < 0:
            idum += im
        j = iy // ndiv
        iy = iv[j]
        iv[j] = idum
        out.append(min(am * iy, rnmx))
    return np.array(out)


def gauss_fields(nx, ny, nz, ncomp, seed):
    """ncomp complex Gaussian fields drawn in the reference's loop order
    (initialize.f90:305-326)."""
    nxh = nx // 2 + 1
    out = np.empty((ncomp, nz, ny, nxh), dtype=np.complex128)
    _ran1_lib().oracle_gauss_fields(nxh, ny, nz, ncomp, seed, out.ctypes.data)
    return out


def initialize_dealiased(nx, ny, nz, seed, akp, u0, kcut, spectrum_kind="akp",
                         kmin=0.0, kmax=0.0):
    """initialize3dvelhighmemdealiased, initialize.f90:284-371.

    spectrum_kind "akp": amplitude u0 sqrt(8 sqrt(2/pi)/(3 pi akp^5)) k
    exp(-k^2/akp^2) (:349).  "kolmogorov": |v| ~ k^(-11/6) on kmin <= k <= kmax
    (E(k) ~ k^(-5/3)), a new initializer that reuses the same draws; both are
    rescaled to E = 3/2 u0^2 (:362-368).
    """
    kx, ky, kz, k2 = wavenumber(nx, ny, nz)
    g = gauss_fields(nx, ny, nz, 3, seed)
    vx, vy, vz = g[0], g[1], g[2]
    KX = np.broadcast_to(kx[None, None, :], k2.shape)
    KY = np.broadcast_to(ky[None, :, None], k2.shape)
    KZ = np.broadcast_to(kz[:, None, None], k2.shape)
    tmpz = KX * vx + KY * vy + KZ * vz                                  # :328-332
    tmpz = tmpz / (KX * KX + KY * KY + KZ * KZ + MYTINY_DP)
    vx = vx - KX * tmpz
    vy = vy - KY * tmpz
    vz = vz - KZ * tmpz
    vx, vy, vz = symmetrize3d(vx), symmetrize3d(vy), symmetrize3d(vz)  # :337-339
    m = k2 >= kcut * kcut                                               # :341-345
    vx, vy, vz = (np.where(m, 0.0, a) for a in (vx, vy, vz))
    if spectrum_kind == "akp":
        tmp = (u0 * np.sqrt(8.0 * np.sqrt(2.0 / PI_REF) / (3.0 * PI_REF * akp ** 5))
               * np.sqrt(k2) * np.exp(-k2 / (akp * akp)))               # :349
    else:
        k = np.sqrt(k2)
        tmp = np.where((k >= kmin) & (k <= kmax), k ** (-11.0 / 6.0), 0.0)
    vx, vy, vz = vx * tmp, vy * tmp, vz * tmp                          # :358-360
    tmp1 = energy((vx, vy, vz))                                        # :362-364
    tmp2 = 1.5 * u0 * u0
    f = np.sqrt(tmp2 / tmp1)
    return f * vx, f * vy, f * vz


# --------------------------------------------------------------------------
# 2D vorticity ensemble member (physics of turb_2d.f90:288-403 and
# spectral_dns_2d.f90:94,160-188, restated; the reference 2D solver itself
# does not run, see spectral_dns_2d.f90:166-168)
# --------------------------------------------------------------------------
@dataclasses.dataclass
class Params2D:
    n: int
    alpha: float = 0.01
    nu8: float = 0.0
    dt: float = 1e-3


def rhs2d(wz, p: Params2D):
    """d(w)/dt nonlinear part: -(i kx (u w)^ + i ky (v w)^), with
    u^ = i ky w^/k2, v^ = -i kx w^/k2 (spectral_dns_2d.f90:161-178), then
    symmetrize2d and the 2/3 mask (:188)."""
    n = p.n
    kx, ky, k2 = wavenumber2d(n, n)
    KX, KY = kx[None, :], ky[:, None]
    const = 1.0 / (n * n)
    u = c2r2(1j * KY * wz / k2, n)
    v = c2r2(-1j * KX * wz / k2, n)
    w = c2r2(wz, n)
    a = r2c(u * w) * const
    b = r2c(v * w) * const
    nl = -(1j * KX * a + 1j * KY * b)
    nl = symmetrize2d(nl)
    nl[k2 >= (2.0 * (n // 2) / 3.0) ** 2] = 0.0
    return nl


def c2r2(c, n):
    return _irfftn(c, (c.shape[0], n), WORKERS)


def if_factor2d(p: Params2D, half=True):
    """E = exp(-(alpha + nu8 k^8) dt/2) (linear damping + hyperviscosity)."""
    _, _, k2 = wavenumber2d(p.n, p.n)
    kk = k2.copy()
    kk[0, 0] = 0.0
    f = 0.5 if half else 1.0
    return np.exp(-(p.alpha + p.nu8 * kk ** 4) * p.dt * f)


def rk4_step2d(wz, p: Params2D):
    """Division-free Lawson IF-RK4 (algebraically dns-deform.f90:160-230)."""
    E = if_factor2d(p)
    dt = p.dt
    k1 = rhs2d(wz, p)
    k2_ = rhs2d(E * (wz + 0.5 * dt * k1), p)
    k3 = rhs2d(E * wz + 0.5 * dt * k2_, p)
    k4 = rhs2d(E * E * wz + E * dt * k3, p)
    return E * E * wz + dt * (E * E * k1 + 2 * E * k2_ + 2 * E * k3 + k4) / 6.0


def initialize2d(n, seed, kpeak=6.0, enstrophy_target=None, energy_target=0.5):
    """Seeded random vorticity with E(k) ~ k exp(-(k/kpeak)^2)
    (draw order of initialize.f90:485-492, then symmetrize2d and the 2/3 mask
    of :494-496); normalised to the given energy."""
    kx, ky, k2 = wavenumber2d(n, n)
    g = gauss_fields(n, n, 1, 1, seed)[0, 0]
    w = symmetrize2d(g)
    w[k2 >= (2.0 * (n // 2) / 3.0) ** 2] = 0.0
    k = np.sqrt(k2)
    # E(k) = pi k |u^|^2 per shell -> |w^| = k |u^| ~ k exp(-(k/kp)^2/2)
    amp = k * np.exp(-0.5 * (k / kpeak) ** 2)
    w = w * amp
    q = (w * np.conj(w)).real / k2
    q[0, 0] = 0.0
    q[:, 0] *= 0.5
    e = float(np.sum(q))
    return w * np.sqrt(energy_target / e)


def energy2d(wz):
    """E = sum |w|^2/k2, 1/2 at kx = 0 (spectral_dns_2d.f90:127-129)."""
    n = wz.shape[0]
    _, _, k2 = wavenumber2d(n, n)
    q = (wz * np.conj(wz)).real / k2
    q[0, 0] = 0.0
    q[:, 0] *= 0.5
    return float(np.sum(q))


# --------------------------------------------------------------------------
# discrete adjoint of the IF-RK4 step (DNS right-hand side)
#
# Gradients are with respect to the real and imaginary parts of every stored
# half-complex entry: g = dJ/dRe(v) + i dJ/dIm(v), so dJ = sum Re(conj(g) dv).
# --------------------------------------------------------------------------
def r2c_T(lam, nx):
    """Transpose of the unnormalised r2c (physical reals -> stored half
    spectrum) under real inner products: 1/2 c2r with the kx = 0 and kx = nx/2
    planes doubled."""
    l = np.array(lam, dtype=np.complex128, copy=True)
    l[..., 0] *= 2.0
    l[..., -1] *= 2.0
    return 0.5 * c2r(l, nx)


def c2r_T(mu):
    """Transpose of the unnormalised c2r: r2c with the interior kx columns
    doubled (the kx = 0 and kx = nx/2 entries enter c2r once, and only through
    their real parts)."""
    X = r2c(mu)
    X[..., 1:-1] *= 2.0
    return X


def symmetrize3d_T(c):
    """Transpose of symmetrize3d (real-linear): the conjugate copies on the
    kx = 0 plane become accumulations into their sources, then the zeroing."""
    c = np.array(c, dtype=np.complex128, copy=True)
    nz, ny, nxh = c.shape
    jz = np.arange(nz // 2 + 1, nz)
    jy = np.arange(ny)
    src_y = np.mod(ny - jy, ny)
    src_z = nz - jz
    jy2 = np.arange(ny // 2 + 1, ny)
    # copies were applied in the order (plane part, then kz = 0 line); undo in reverse
    c[0, ny - jy2, 0] += np.conj(c[0, jy2, 0])
    c[0, jy2, 0] = 0.0
    tgt = c[jz[:, None], jy[None, :], 0].copy()
    np.add.at(c, (src_z[:, None].repeat(ny, 1), src_y[None, :].repeat(len(jz), 0), 0), np.conj(tgt))
    c[jz[:, None], jy[None, :], 0] = 0.0
    c[:, ny // 2, :] = 0.0
    c[nz // 2, :, :] = 0.0
    c[:, :, nxh - 1] = 0.0
    c[0, 0, 0] = 0.0
    return c


def cross(a, b):
    return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])


def ratesdudt_adj(s, lam_w, grid: Grid):
    """lam_s = R'(s)^T lam_w for the DNS right-hand side of ratesdudt."""
    p = grid.p
    kx, ky, kz, k2 = grid.kx, grid.ky, grid.kz, grid.k2
    nx, ny, nz = p.nx, p.ny, p.nz
    N3 = float(nx * ny * nz)
    mu = list(projection(*lam_w, kx, ky, kz))
    if p.mask == "rhs_and_step":
        m = k2 >= p.kcut * p.kcut
        mu = [np.where(m, 0.0, a) for a in mu]
    mu = [symmetrize3d_T(a) for a in mu]
    lam = [np.zeros_like(a) for a in s]
    if p.forced:
        kf = forcing_energy(*s, k2, p.fkmax)
        a = p.eps / (2.0 * kf)
        m = k2 < p.fkmax * p.fkmax
        c = sum(float(np.sum(np.where(m, (np.conj(x) * y).real, 0.0))) for x, y in zip(mu, s))
        w = np.ones(k2.shape)
        w[:, :, 0] = 0.5
        lam = [l + np.where(m, a * x - (a * c / kf) * 2.0 * w * y, 0.0) for l, x, y in zip(lam, mu, s)]
    u = [c2r(a, nx) for a in s]
    om = [c2r(a, nx) for a in vorticity(*s, kx, ky, kz)]
    phi = [r2c_T(a, nx) / N3 for a in mu]
    au = cross(om, phi)
    aw = cross(phi, u)
    gu = [c2r_T(a) for a in au]
    gw = vorticity(*[c2r_T(a) for a in aw], kx, ky, kz)   # the curl is self-adjoint
    return [l + x + y for l, x, y in zip(lam, gu, gw)]


def rk4_step_adj(v, lam_next, grid: Grid):
    """lam_n = S'(v_n)^T lam_{n+1} for one IF-RK4 step in the division-free
    form v' = M[E^2 v + (E^2 dt w1 + 2E dt w2 + 2E dt w3 + dt w4)/6]."""
    p = grid.p
    dt = p.dt
    E = np.exp(-p.nu * grid.k2 * dt / 2)
    s1 = list(v)
    w1 = ratesdudt(s1, grid)
    s2 = [E * a + 0.5 * dt * E * b for a, b in zip(v, w1)]
    w2 = ratesdudt(s2, grid)
    s3 = [E * a + 0.5 * dt * b for a, b in zip(v, w2)]
    w3 = ratesdudt(s3, grid)
    s4 = [E * E * a + E * dt * b for a, b in zip(v, w3)]
    m = grid.k2 >= p.kcut * p.kcut
    lt = [np.where(m, 0.0, a) for a in lam_next]
    lv = [E * E * a for a in lt]
    lw = [dt / 6.0 * a for a in lt]
    ls = ratesdudt_adj(s4, lw, grid)
    lv = [x + E * E * y for x, y in zip(lv, ls)]
    lw = [2 * E * dt / 6.0 * a + E * dt * b for a, b in zip(lt, ls)]
    ls = ratesdudt_adj(s3, lw, grid)
    lv = [x + E * y for x, y in zip(lv, ls)]
    lw = [2 * E * dt / 6.0 * a + 0.5 * dt * b for a, b in zip(lt, ls)]
    ls = ratesdudt_adj(s2, lw, grid)
    lv = [x + E * y for x, y in zip(lv, ls)]
    lw = [E * E * dt / 6.0 * a + 0.5 * E * dt * b for a, b in zip(lt, ls)]
    ls = ratesdudt_adj(s1, lw, grid)
    return [x + y for x, y in zip(lv, ls)]


def rk4_step_lawson(v, grid: Grid):
    """The division-free form of rk4_step (the map rk4_step_adj transposes)."""
    p = grid.p
    dt = p.dt
    E = np.exp(-p.nu * grid.k2 * dt / 2)
    w1 = ratesdudt(v, grid)
    w2 = ratesdudt([E * a + 0.5 * dt * E * b for a, b in zip(v, w1)], grid)
    w3 = ratesdudt([E * a + 0.5 * dt * b for a, b in zip(v, w2)], grid)
    w4 = ratesdudt([E * E * a + E * dt * b for a, b in zip(v, w3)], grid)
    out = [E * E * a + dt * (E * E * b + 2 * E * c + 2 * E * d + e) / 6.0
           for a, b, c, d, e in zip(v, w1, w2, w3, w4)]
    return mask_state(out, grid)


def shell_mask(k2, kmin, kmax):
    ll = np.floor(np.sqrt(k2) + 0.5)
    return (ll >= kmin) & (ll <= kmax)


def shell_enstrophy(v, k2, kmin=8, kmax=16):
    """J = sum over shells kmin..kmax of k^2 q(k) (q = 1/2-weighted |v|^2 at kx = 0)."""
    m = shell_mask(k2, kmin, kmax)
    q = _q(v)
    return float(np.sum(np.where(m, k2 * q, 0.0)))


def shell_enstrophy_grad(v, k2, kmin=8, kmax=16):
    m = shell_mask(k2, kmin, kmax)
    w = np.ones(k2.shape)
    w[:, :, 0] = 0.5
    return [np.where(m, 2.0 * w * k2 * a, 0.0) for a in v]


def adjoint_gradient(v0, grid: Grid, nsteps, kmin=8, kmax=16, checkpoint=0):
    """dJ/dv0 for J = shell_enstrophy(v_T) after nsteps Lawson IF-RK4 steps,
    with checkpoints every `checkpoint` steps (0: keep every state)."""
    K = checkpoint or nsteps
    cps = {0: [a.copy() for a in v0]}
    v = list(v0)
    for n in range(nsteps):
        v = rk4_step_lawson(v, grid)
        if (n + 1) % K == 0 and n + 1 < nsteps:
            cps[n + 1] = [a.copy() for a in v]
    lam = shell_enstrophy_grad(v, grid.k2, kmin, kmax)
    for seg in range((nsteps - 1) // K, -1, -1):
        n0 = seg * K
        n1 = min(nsteps, n0 + K)
        states = [cps[n0]]
        for n in range(n0, n1 - 1):
            states.append(rk4_step_lawson(states[-1], grid))
        for n in range(n1 - 1, n0 - 1, -1):
            lam = rk4_step_adj(states[n - n0], lam, grid)
    return lam, shell_enstrophy(v, grid.k2, kmin, kmax)
