"""Threaded CPU restatement of the forced-DNS IF-RK4 step, for timing.

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` and the CPU-baseline / reference
legs of ``bench.py`` may use this module.  It is the timed CPU baseline: the
same arithmetic as ``spectral_ref.rk4_step`` (dns-deform.f90:160-237 over
the right-hand side of dns-deform.f90:259-288: vorticity, convec_dns.f90,
force.f90, symmetrize.f90:32-64, projection.f90, the 2/3 mask), organised
so that every host core works: the 3D transforms run in scipy.fft with
``workers`` threads, and every pointwise pass runs over z-slabs of the
fields in a thread pool (NumPy releases the interpreter lock inside its
array loops).  ``tests/test_oracle_pins.py`` checks it against
``spectral_ref.rk4_step``.

Two precisions, as the reference builds in two: ``np.complex128`` follows
constant.f90 (kind sp = double), ``np.complex64`` follows constant_sp.f90
(kind sp = single; mytiny = tiny(1.0_sp), constant_sp.f90:15).  The forcing's
band energy K_f is summed in double in both.
"""
from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from oracle import spectral_ref as R


class CpuRK4:
    """One forced-DNS grid: IF-RK4 steps of a state held as three spectral
    fields of shape (nz, ny, nx/2+1)."""

    def __init__(self, grid: R.Grid, workers: int, dtype=np.complex128):
        p = grid.p
        self.p, self.workers = p, max(1, int(workers))
        self.cdt = np.dtype(dtype)
        self.rdt = np.float32 if self.cdt == np.complex64 else np.float64
        self.tiny = R.MYTINY_SP if self.cdt == np.complex64 else R.MYTINY_DP
        self.kx = grid.kx.astype(self.rdt)
        self.ky = grid.ky.astype(self.rdt)
        self.kz = grid.kz.astype(self.rdt)
        nz, ny, nxh = p.nz, p.ny, p.nx // 2 + 1
        self.shape = (nz, ny, nxh)
        # dns-deform.f90:90, k2e = exp(-nu k2 dt / 2) stored as a 3D array
        self.k2e = np.exp(-p.nu * grid.k2 * p.dt / 2).astype(self.rdt)
        nchunk = min(nz, 4 * self.workers)
        edges = np.linspace(0, nz, nchunk + 1).astype(int)
        self.chunks = [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]
        self.pool = ThreadPoolExecutor(self.workers) if self.workers > 1 else None
        kb = int(math.ceil(p.fkmax))
        self.band_z = np.unique(np.r_[0:min(kb + 1, nz), max(nz - kb, 0):nz])
        self.band_y = np.unique(np.r_[0:min(kb + 1, ny), max(ny - kb, 0):ny])
        self.band_x = np.arange(min(kb + 1, nxh))
        k2b = (grid.kz[self.band_z][:, None, None] ** 2 + grid.ky[self.band_y][None, :, None] ** 2
               + grid.kx[self.band_x][None, None, :] ** 2)
        k2b[(self.band_z == 0)[:, None, None] & (self.band_y == 0)[None, :, None]
            & (self.band_x == 0)[None, None, :]] = R.MYTINY_SP
        self.band_mask = k2b < p.fkmax * p.fkmax          # force.f90: k2 < fkmax^2
        self.band_weight = np.where(self.band_x == 0, 0.5, 1.0)[None, None, :]
        self.kcut2 = p.kcut * p.kcut
        self.w = [np.empty(self.shape, self.cdt) for _ in range(3)]
        self.du = [np.empty(self.shape, self.cdt) for _ in range(3)]
        self.s = [np.empty(self.shape, self.cdt) for _ in range(3)]

    def close(self):
        if self.pool is not None:
            self.pool.shutdown()
            self.pool = None

    # -- helpers -----------------------------------------------------------
    def _each(self, fn):
        if self.pool is None:
            for c in self.chunks:
                fn(*c)
        else:
            list(self.pool.map(lambda c: fn(*c), self.chunks))

    def _k(self, z0, z1):
        return self.kx[None, None, :], self.ky[None, :, None], self.kz[z0:z1, None, None]

    def _symmetrize(self, c):
        """symmetrize.f90:32-64 in place (zero the Nyquist planes and the mean
        mode, then the kx = 0 conjugate copies)."""
        nz, ny, nxh = c.shape
        c[:, ny // 2, :] = 0.0
        c[nz // 2, :, :] = 0.0
        c[:, :, nxh - 1] = 0.0
        c[0, 0, 0] = 0.0
        plane = c[:, :, 0]
        jz = np.arange(nz // 2 + 1, nz)
        src_y = np.mod(ny - np.arange(ny), ny)
        plane[jz, :] = np.conj(plane[nz - jz][:, src_y])
        jy2 = np.arange(ny // 2 + 1, ny)
        plane[0, jy2] = np.conj(plane[0, ny - jy2])

    # -- the right-hand side (dns-deform.f90:259-288) -----------------------
    def rhs(self, v):
        p, w = self.p, self.w
        vx, vy, vz = v
        nx, ny, nz = p.nx, p.ny, p.nz

        def vort(z0, z1):                                   # dns-deform.f90:265-273
            KX, KY, KZ = self._k(z0, z1)
            a, b, c = vx[z0:z1], vy[z0:z1], vz[z0:z1]
            w[0][z0:z1] = 1j * (KY * c - KZ * b)
            w[1][z0:z1] = 1j * (KZ * a - KX * c)
            w[2][z0:z1] = 1j * (KX * b - KY * a)

        self._each(vort)
        s = (nz, ny, nx)
        u = [R._irfftn(a, s, self.workers) for a in v]        # convec_dns.f90:22-27
        o = [R._irfftn(a, s, self.workers) for a in w]
        const = self.rdt(1.0 / float(nx * ny * nz))            # convec_dns.f90:15

        def cross(z0, z1):                                  # convec_dns.f90:30-42
            ux, uy, uz = (a[z0:z1] for a in u)
            ox, oy, oz = (a[z0:z1] for a in o)
            lx = uy * oz - uz * oy
            ly = uz * ox - ux * oz
            lz = ux * oy - uy * ox
            ox[...] = lx * const
            oy[...] = ly * const
            oz[...] = lz * const

        self._each(cross)
        for i in range(3):                                  # convec_dns.f90:45-47
            w[i] = R._rfftn(o[i], self.workers)
        del u, o
        if p.forced:                                        # force.f90:3-31
            ix = np.ix_(self.band_z, self.band_y, self.band_x)
            sub = [a[ix].astype(np.complex128) for a in v]
            q = sum((a * np.conj(a)).real for a in sub) * self.band_weight
            kinet = float(np.sum(np.where(self.band_mask, q, 0.0)))
            amp = p.eps / (2.0 * kinet)
            for i in range(3):
                wi = w[i][ix]
                w[i][ix] = np.where(self.band_mask, wi + (amp * sub[i]).astype(self.cdt), wi)
        for i in range(3):                                  # dns-deform.f90:281-283
            self._symmetrize(w[i])
        tiny = self.rdt(self.tiny)

        def proj(z0, z1):                                   # projection.f90:2-31
            KX, KY, KZ = self._k(z0, z1)
            a, b, c = w[0][z0:z1], w[1][z0:z1], w[2][z0:z1]
            t = (KX * a + KY * b + KZ * c) / (KX * KX + KY * KY + KZ * KZ + tiny)
            a -= KX * t
            b -= KY * t
            c -= KZ * t

        self._each(proj)
        return w

    # -- one IF-RK4 step (dns-deform.f90:160-237) ---------------------------
    def step(self, v):
        """Advance v (three arrays of dtype, updated in place) by one step."""
        dt = self.rdt(self.p.dt)
        du, st, k2e = self.du, self.s, self.k2e
        for stage in range(4):
            w = self.rhs(v if stage == 0 else st)

            def upd(z0, z1, stage=stage):
                e = k2e[z0:z1]
                for i in range(3):
                    vi, wi, di, si = v[i][z0:z1], w[i][z0:z1], du[i][z0:z1], st[i][z0:z1]
                    if stage == 0:                          # :164-179
                        ku = dt * wi
                        di[...] = ku
                        si[...] = e * (vi + ku / 2)
                    elif stage < 3:                         # :182-196 and :199-213
                        ku = dt * wi / e
                        di += 2 * ku
                        si[...] = e * (vi + ku / 2) if stage == 1 else e * e * (vi + ku)
                    else:                                   # :216-228
                        ku = dt * wi / e / e
                        di += ku
                        vi[...] = e * e * (vi + di / 6)
                if stage == 3:                              # :233-237 the 2/3 mask
                    KX, KY, KZ = self._k(z0, z1)
                    m = (KX * KX + KY * KY + KZ * KZ) >= self.kcut2
                    for i in range(3):
                        v[i][z0:z1][m] = 0.0

            self._each(upd)
        return v
