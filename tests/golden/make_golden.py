"""Generate the golden fixtures under tests/golden/ from the FP64 oracle.

    python tests/golden/make_golden.py

Fixtures (NumPy .npz, complex128 spectral fields in the reference layout
(nz, ny, nx/2+1)): the seeded 16^3 initial field (ran1 seed 1, akp = 4,
E = 0.5), its right-hand side, the state after 1 and 10 IF-RK4 steps, after
3 IF-AB2 passes, and the Smagorinsky / dynamic-Smagorinsky stresses.  c1_128:
the forced-DNS configuration at 128^3 in FP64 (nu = 0.01, dt = 2e-3, the same
seeded field) after 1, 10 and 100 steps, stored compactly as the block of
wavenumbers |kx|, |ky|, |kz| <= 6 plus, after 100 steps, the shell spectrum,
energy and dissipation (python tests/golden/make_golden.py c1; a few minutes).
schemes16: from the same 16^3 field, the rotating solver after 5 passes
(om = 5, band forcing 1 <= |k| < 2.5), the same with a passive scalar (a
seeded dealiased white-noise phi, pr = 0.7, scalar forcing on) and the
variable-step IF-AB2 after 6 uneven steps (cut at k >= nx/2), and the
variable-step scalar solver after the same steps (mean-gradient forcing, the
history as written) (python tests/golden/make_golden.py schemes).  The
reference itself cannot be run here; these fixtures freeze the oracle's
outputs so that both the oracle and the CUDA library are checked against the
same committed numbers.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import spectral_ref as R  # noqa: E402

N = 16
NU, DT = 0.01, 2e-3


def main():
    kcut = 2.0 * (N // 2) / 3.0
    v0 = R.initialize_dealiased(N, N, N, 1, 4.0, 1.0 / np.sqrt(3.0), kcut)
    g = R.Grid(R.Params(nx=N, nu=NU, dt=DT))
    w0 = R.ratesdudt(v0, g)
    v1 = R.rk4_run(v0, g, 1)
    v10 = R.rk4_run(v0, g, 10)
    vab, _ = R.ab2_run(v0, g, 3)
    kx, ky, kz, k2 = R.wavenumber(N, N, N)
    delta = R.PI_REF / kcut
    ts = R.smag(*v0, kx, ky, kz, N, delta, 0.0289)
    td, mm, lm, cs2 = R.dynsmag(*v0, kx, ky, kz, R.test_filter(k2, kcut / 2), N, delta, 2 * delta, True, 0.0)
    np.savez_compressed(os.path.join(HERE, "dns16.npz"), v0=np.stack(v0), w0=np.stack(w0), v1=np.stack(v1),
                        v10=np.stack(v10), vab3=np.stack(vab), nu=NU, dt=DT, n=N)
    np.savez_compressed(os.path.join(HERE, "les16.npz"), tau_smag=np.stack(ts), tau_dyn=np.stack(td),
                        mm=mm, lm=lm, cs2=cs2, c1=0.0289, delta=delta, n=N)
    np.savez_compressed(os.path.join(HERE, "ran1_seed1.npz"), seq=R.ran1_sequence(1, 4096),
                        seq_m7=R.ran1_sequence(-7, 4096))


C1_N, C1_K = 128, 6


def c1_block(v):
    """Wavenumbers |kx|, |ky|, |kz| <= C1_K of three (nz, ny, nx/2+1) fields."""
    idx = np.r_[0:C1_K + 1, C1_N - C1_K:C1_N]
    return np.stack([a[np.ix_(idx, idx, np.arange(C1_K + 1))] for a in v])


def c1():
    n = C1_N
    kcut = 2.0 * (n // 2) / 3.0
    v = R.initialize_dealiased(n, n, n, 1, 4.0, 1.0 / np.sqrt(3.0), kcut)
    g = R.Grid(R.Params(nx=n, nu=NU, dt=DT))
    out = {}
    done = 0
    for target in (1, 10, 100):
        v = R.rk4_run(v, g, target - done)
        done = target
        out["v%d" % target] = c1_block(v)
    _, _, _, k2 = R.wavenumber(n, n, n)
    out["ek100"] = R.spectrum(v, k2, n)
    out["energy100"] = R.energy(v)
    out["diss100"] = R.dissipation(v, k2, NU)
    np.savez_compressed(os.path.join(HERE, "c1_128.npz"), n=n, kmax=C1_K, nu=NU, dt=DT, **out)


STEPS_V = [2e-3, 2.6e-3, 1.4e-3, 2.2e-3, 1.8e-3, 2.4e-3]


def schemes():
    kcut = 2.0 * (N // 2) / 3.0
    v0 = R.initialize_dealiased(N, N, N, 1, 4.0, 1.0 / np.sqrt(3.0), kcut)
    g = R.Grid(R.Params(nx=N, nu=NU, dt=DT, forced=True, eps=0.1))
    v_rot, _, _ = R.rot_run(v0, g, 5, 5.0, 1.0, 2.5)
    rng = np.random.default_rng(7)
    phi0 = R.dealiasing(R.r2c(rng.standard_normal((N, N, N))) / N ** 3, g.k2)
    v_rs, phi_rs, _, _ = R.rot_scalar_run(v0, phi0, g, 5, 5.0, 1.0, 2.5, 0.7, True, 0.05)
    gv = R.Grid(R.Params(nx=N, nu=NU, forced=True, eps=0.1, kcut=N // 2))
    v_ab2v, t, dto = R.ab2v_run(v0, gv, STEPS_V)
    phis = R.symmetrize3d(phi0)
    v_vs, phi_vs, _, _ = R.ab2v_scalar_run(v0, phis, g, STEPS_V, 0.7, True, 0.3)
    np.savez_compressed(os.path.join(HERE, "schemes16.npz"), v0=np.stack(v0), v_rot5=np.stack(v_rot),
                        phi0=phi0, v_rs5=np.stack(v_rs), phi_rs5=phi_rs, v_ab2v=np.stack(v_ab2v),
                        steps_v=np.array(STEPS_V), t_ab2v=t, dto_ab2v=dto, v_vs=np.stack(v_vs),
                        phi_vs=phi_vs, n=N, nu=NU, dt=DT)


if __name__ == "__main__":
    if sys.argv[1:] == ["c1"]:
        c1()
    elif sys.argv[1:] == ["schemes"]:
        schemes()
    else:
        main()
