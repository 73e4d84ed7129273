"""Shared helpers for the parity tests (seeded inputs, error norms)."""
import numpy as np

from oracle import spectral_ref as R


def rel_l2(a, b):
    """Relative L2 error of a against the reference b, over all fields."""
    a = list(a) if isinstance(a, (list, tuple)) else [a]
    b = list(b) if isinstance(b, (list, tuple)) else [b]
    num = sum(float(np.sum(np.abs(np.asarray(x, np.complex128) - np.asarray(y)) ** 2))
              for x, y in zip(a, b))
    den = sum(float(np.sum(np.abs(np.asarray(y)) ** 2)) for y in b)
    return float(np.sqrt(num / den)) if den > 0 else float(np.sqrt(num))


def fresh(a, dtype):
    """A new C-contiguous array of `dtype` holding a's values.  Every buffer
    handed to an in-place GPU call is made this way: np.ascontiguousarray
    returns its argument itself when the dtype already matches, and an
    in-place call would then also change the array the reference result is
    computed from."""
    return np.array(a, dtype=dtype, order="C", copy=True)


def hermitian_fields(shape, seed, ncomp=3, kcut=None):
    """Spectral fields of seeded real white-noise physical fields (so every
    kx = 0 / Nyquist symmetry is exact), shape = (nx, ny, nz)."""
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    out = [R.r2c(rng.standard_normal((nz, ny, nx))) / (nx * ny * nz) for _ in range(ncomp)]
    if kcut is not None:
        _, _, _, k2 = R.wavenumber(nx, ny, nz)
        out = [np.where(k2 >= kcut * kcut, 0.0, a) for a in out]
    return out


def complex_noise(shape, seed, ncomp=3):
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    s = (nz, ny, nx // 2 + 1)
    return [rng.standard_normal(s) + 1j * rng.standard_normal(s) for _ in range(ncomp)]


def solenoidal_init(n, seed=1, akp=4.0, u0=1.0 / np.sqrt(3.0)):
    return R.initialize_dealiased(n, n, n, seed, akp, u0, 2.0 * (n // 2) / 3.0)
