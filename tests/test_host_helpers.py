"""Host-side checks of arithmetic helpers the kernels share: the integer
forms of real wavenumber bounds (k2_lt, k2_le), the exact shell index
floor(sqrt(k2) + 1/2), the incremental grid-stride index walk (Walk3) and the
compile-time roots of unity of the warp FFT.  A small host program is built
against the kernel headers with nvcc and run on the CPU (no GPU needed)."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "speccodelib_gb300", "csrc")

PROGRAM = r'''
#include <cstdio>
#include <cmath>
#include "sc_xwarp.cuh"
int main() {
  // k2_lt / k2_le against the real comparisons, k2 in [0, 4000]
  const double ts[] = {-1.0, 0.0, 0.25, 1.0, 2.5, 6.25, 7.0, 7.000001, 113.77777777777777, 1024.0, 1e30};
  for (double t : ts) {
    const int lt = sc::k2_lt(t), le = sc::k2_le(t);
    for (int k2 = 0; k2 <= 4000; ++k2) {
      if ((k2 < lt) != ((double)k2 < t)) { std::printf("lt %g %d\n", t, k2); return 1; }
      if ((k2 < le) != ((double)k2 <= t)) { std::printf("le %g %d\n", t, k2); return 1; }
    }
  }
  // shell index: every k2 up to 3 * 2048^2 (ny, nz up to 4096 at kx = 2048)
  for (int k2 = 0; k2 <= 3 * 2048 * 2048; ++k2) {
    const long long n = sc::shell_index(k2);
    if (!(n * n - n < k2 || k2 == 0) || !(k2 <= n * n + n)) { std::printf("shell %d %lld\n", k2, n); return 1; }
  }
  // Walk3 against direct division, odd strides and extents
  const int ns[] = {1, 7, 257, 33}, nys[] = {1, 5, 512, 3};
  const long long strides[] = {1, 3, 256, 311296, 1000003};
  for (int a = 0; a < 4; ++a)
    for (long long st : strides) {
      const int n = ns[a], ny = nys[a];
      const long long total = (long long)n * ny * 11;
      for (long long t0 = 0; t0 < 5; ++t0)
        for (sc::Walk3 w(t0, st, total, n, ny); w.ok(); w.next()) {
          const long long r = w.t / n;
          if (w.ix != w.t % n || w.iy != r % ny || w.iz != r / ny || w.row() != r) {
            std::printf("walk %d %d %lld %lld\n", n, ny, st, w.t); return 1;
          }
        }
    }
  // roots of unity used as compile-time twiddles: cos, sin of 2 pi j / n
  for (int n = 8; n <= 64; n *= 2)
    for (int j = 0; j < n; ++j) {
      const double c = sc::roots::cos2pi(j, n, false), s = sc::roots::cos2pi(j, n, true);
      std::printf("%d %d %.17g %.17g\n", n, j, c, s);
    }
  return 0;
}
'''


@pytest.fixture(scope="module")
def helper_output(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    d = tmp_path_factory.mktemp("helpers")
    src = d / "helpers.cu"
    src.write_text(PROGRAM)
    exe = d / "helpers"
    cmd = [nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", CSRC, str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-500:]
    return r.stdout


def test_bounds_shells_and_walk(helper_output):
    """k2_lt, k2_le, shell_index and Walk3 hold for every case the program
    checks (it exits non-zero at the first failure)."""
    assert helper_output.strip()


def test_compile_time_roots(helper_output):
    """The compile-time cos / sin of 2 pi j / n are within 2 ulp of the
    correctly rounded values (numpy's, from long double)."""
    for line in helper_output.strip().splitlines():
        n, j, c, s = line.split()
        n, j = int(n), int(j)
        x = 2 * np.pi * np.longdouble(j) / n
        rc, rs = float(np.cos(x)), float(np.sin(x))
        assert abs(float(c) - rc) <= 2 * np.spacing(1.0) * max(1.0, abs(rc))
        assert abs(float(s) - rs) <= 2 * np.spacing(1.0) * max(1.0, abs(rs))


ROT_PROGRAM = r'''
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "sc_common.cuh"
#include "sc_rot.cuh"
// Reads: int nx, ny, nz, npasses, scalar; double nu, dt, om, kcut2, pr; v0
// (3 fields) [phi0 (1 field) when scalar], then per pass the right-hand side
// (3 fields) [and wphi (1 field)], complex128 (nz, ny, nx/2+1).  Writes, for
// T = double then float, v [and phi] after every pass (complex128).  With a
// scalar the rebuilt velocity is not truncated, as in rot_update_kernel.
template <typename T>
static void run(const int* hd, const double* sc, const std::vector<double>& in0, const std::vector<double>& ws,
                FILE* out) {
  const int nx = hd[0], ny = hd[1], nz = hd[2], np = hd[3], scalar = hd[4];
  const int nf = scalar ? 4 : 3;
  const long long nxh = nx / 2 + 1, field = (long long)nz * ny * nxh;
  std::vector<sc::Cx<T>> f(nf * field), o(3 * field), a(2 * field), op(field), p0(field);
  for (long long i = 0; i < nf * field; ++i) f[i] = sc::cx((T)in0[2 * i], (T)in0[2 * i + 1]);
  const int kc = sc::k2_lt(sc[3]);
  for (int p = 0; p < np; ++p) {
    const double* w = ws.data() + (size_t)p * 2 * nf * field;
    for (int iz = 0; iz < nz; ++iz)
      for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nxh; ++ix) {
          const long long idx = ((long long)iz * ny + iy) * nxh + ix;
          const int ky = iy < ny / 2 ? iy : iy - ny, kz = iz < nz / 2 ? iz : iz - nz;
          const int k2 = ix * ix + ky * ky + kz * kz;
          sc::Cx<T> vv[3], ww[3], oo[3];
          for (int c = 0; c < 3; ++c) {
            vv[c] = f[c * field + idx];
            oo[c] = o[c * field + idx];
            ww[c] = sc::cx((T)w[2 * (c * field + idx)], (T)w[2 * (c * field + idx) + 1]);
          }
          sc::rot_point<T>(p < 2 ? p : 2, ix, ky, kz, !scalar && k2 >= kc, (T)sc[0], (T)sc[1], (T)sc[2], vv, ww, oo,
                           a[idx], a[field + idx]);
          for (int c = 0; c < 3; ++c) { f[c * field + idx] = vv[c]; o[c * field + idx] = oo[c]; }
          if (scalar) {
            const sc::Cx<T> wp = sc::cx((T)w[2 * (3 * field + idx)], (T)w[2 * (3 * field + idx) + 1]);
            sc::rot_scalar_point<T>(p < 2 ? p : 2, k2, (T)sc[0], (T)sc[1], (T)sc[4], f[3 * field + idx], wp,
                                    op[idx], p0[idx]);
          }
        }
    for (long long i = 0; i < nf * field; ++i) {
      const double z[2] = {(double)f[i].re, (double)f[i].im};
      fwrite(z, sizeof(double), 2, out);
    }
  }
}
int main(int argc, char** argv) {
  FILE* in = fopen(argv[1], "rb");
  FILE* out = fopen(argv[2], "wb");
  if (!in || !out) return 2;
  int hd[5];
  double sc[5];
  if (fread(hd, sizeof(int), 5, in) != 5 || fread(sc, sizeof(double), 5, in) != 5) return 3;
  const int nf = hd[4] ? 4 : 3;
  const long long field = (long long)hd[2] * hd[1] * (hd[0] / 2 + 1);
  std::vector<double> in0(2 * nf * field), ws((size_t)hd[3] * 2 * nf * field);
  if (fread(in0.data(), sizeof(double), in0.size(), in) != in0.size()) return 4;
  if (fread(ws.data(), sizeof(double), ws.size(), in) != ws.size()) return 5;
  run<double>(hd, sc, in0, ws, out);
  run<float>(hd, sc, in0, ws, out);
  fclose(out);
  return 0;
}
'''


def _run_rot_program(tmp_path, n, npass, header_d, start, per_pass):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "rot.cu"
    src.write_text(ROT_PROGRAM)
    exe = tmp_path / "rot"
    cmd = [nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", CSRC, str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    nf = len(start)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        f.write(np.array([n, n, n, npass, 1 if nf == 4 else 0], np.int32).tobytes())
        f.write(np.array(header_d, np.float64).tobytes())
        f.write(np.ascontiguousarray(np.stack(start), np.complex128).tobytes())
        for fields in per_pass:
            f.write(np.ascontiguousarray(np.stack(fields), np.complex128).tobytes())
    r = subprocess.run([str(exe), str(fin), str(fout)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-500:]
    return np.fromfile(fout, np.complex128).reshape(2, npass, nf, n, n, n // 2 + 1)


@pytest.mark.parametrize("om", [0.0, 40.0, 900.0])
def test_rotating_update_matches_oracle(tmp_path, om):
    """The per-mode helical-wave AB2 update that rot_update_kernel runs
    (rot_point, sc_rot.cuh), compiled for the host, reproduces the oracle's
    rotating solver pass by pass when fed the oracle's own right-hand sides:
    FP64 to 1e-13, FP32 to 1e-5 (relative L2).  om = 900 at dt = 2e-3 puts
    the inertial-wave phase 2 dt kz om / |k| past pi, where the principal
    square root of the integrating factor matters."""
    from oracle import spectral_ref as R
    from _util import rel_l2, solenoidal_init
    n, npass = 16, 4
    g = R.Grid(R.Params(nx=n, nu=0.01, dt=2e-3, forced=True, eps=0.1))
    v0 = solenoidal_init(n)
    trace = []
    R.rot_run(v0, g, npass, om, 1.0, 2.5, trace=trace)
    kcut2 = (2.0 * (n // 2) / 3.0) ** 2
    out = _run_rot_program(tmp_path, n, npass, [g.p.nu, g.p.dt, om, kcut2, 1.0], list(v0),
                           [list(w) for w, _ in trace])
    for p, (_, vref) in enumerate(trace):
        assert rel_l2(list(out[0, p]), list(vref)) < 1e-13, p
        assert rel_l2(list(out[1, p]), list(vref)) < 1e-5, p


def test_rotating_scalar_update_matches_oracle(tmp_path):
    """The same with the passive scalar of spectral_rot_dns_scalar_ft.f90
    (rot_scalar_point; velocity not truncated after the update), scalar
    forcing on: velocity and scalar pass by pass."""
    from oracle import spectral_ref as R
    from _util import hermitian_fields, rel_l2, solenoidal_init
    n, npass, om, pr = 16, 4, 40.0, 0.7
    g = R.Grid(R.Params(nx=n, nu=0.01, dt=2e-3, forced=True, eps=0.1))
    v0 = solenoidal_init(n)
    phi0 = R.dealiasing(hermitian_fields((n, n, n), 7, ncomp=1)[0], g.k2)
    trace = []
    R.rot_scalar_run(v0, phi0, g, npass, om, 1.0, 2.5, pr, True, 0.05, trace=trace)
    out = _run_rot_program(tmp_path, n, npass, [g.p.nu, g.p.dt, om, 0.0, pr], list(v0) + [phi0],
                           [list(w) + [wphi] for w, wphi, _, _ in trace])
    for p, (_, _, vref, pref) in enumerate(trace):
        assert rel_l2(list(out[0, p, :3]), list(vref)) < 1e-13, p
        assert rel_l2(out[0, p, 3], pref) < 1e-13, p
        assert rel_l2(list(out[1, p, :3]), list(vref)) < 1e-5, p
        assert rel_l2(out[1, p, 3], pref) < 1e-5, p


AB2V_PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "sc_common.cuh"
#include "sc_ab2v.cuh"
// Reads: int nx, ny, nz, npasses, scalar, hist_rhs; double nu, kcut2, pr;
// npasses steps dt; v0 (3 fields) [phi0 when scalar], then per pass the
// right-hand side (3 fields) [and wphi], complex128 (nz, ny, nx/2+1).
// Writes, for T = double then float, v [and phi] after every pass, with the
// weights and the dto bookkeeping of the library's ab2v_pass; with a scalar
// the velocity is not truncated, as in ab2v_update_kernel.
template <typename T>
static void run(const int* hd, const double* sc, const std::vector<double>& dts, const std::vector<double>& in0,
                const std::vector<double>& ws, FILE* out) {
  const int nx = hd[0], ny = hd[1], nz = hd[2], np = hd[3], scalar = hd[4], hist = hd[5];
  const int nf = scalar ? 4 : 3;
  const long long nxh = nx / 2 + 1, field = (long long)nz * ny * nxh;
  std::vector<sc::Cx<T>> f(nf * field), o(3 * field), v0(3 * field), op(field), p0(field);
  for (long long i = 0; i < nf * field; ++i) f[i] = sc::cx((T)in0[2 * i], (T)in0[2 * i + 1]);
  const int kc = sc::k2_lt(sc[1]);
  double dto = 0.0;
  for (int p = 0; p < np; ++p) {
    const double dt = dts[p];
    double s, ek, dl;
    sc::ab2v_weights(p, dt, dto, s, ek, dl);
    const double* w = ws.data() + (size_t)p * 2 * nf * field;
    for (int iz = 0; iz < nz; ++iz)
      for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nxh; ++ix) {
          const long long idx = ((long long)iz * ny + iy) * nxh + ix;
          const int ky = iy < ny / 2 ? iy : iy - ny, kz = iz < nz / 2 ? iz : iz - nz;
          const int k2 = ix * ix + ky * ky + kz * kz;
          sc::Cx<T> vv[3], ww[3], oo[3], zz[3];
          for (int c = 0; c < 3; ++c) {
            vv[c] = f[c * field + idx];
            oo[c] = o[c * field + idx];
            zz[c] = v0[c * field + idx];
            ww[c] = sc::cx((T)w[2 * (c * field + idx)], (T)w[2 * (c * field + idx) + 1]);
          }
          sc::ab2v_point<T>(p < 2 ? p : 2, k2, !scalar && (k2 >= kc || k2 == 0), (T)sc[0], (T)dt, (T)dto, (T)s,
                            (T)ek, (T)dl, vv, ww, oo, zz);
          for (int c = 0; c < 3; ++c) {
            f[c * field + idx] = vv[c];
            o[c * field + idx] = oo[c];
            v0[c * field + idx] = zz[c];
          }
          if (scalar) {
            const sc::Cx<T> wp = sc::cx((T)w[2 * (3 * field + idx)], (T)w[2 * (3 * field + idx) + 1]);
            sc::ab2v_scalar_point<T>(p < 2 ? p : 2, k2, hist != 0, (T)sc[0], (T)dt, (T)dto, (T)sc[2], (T)s, (T)ek,
                                     (T)dl, f[3 * field + idx], wp, op[idx], p0[idx]);
          }
        }
    dto = p == 1 ? dt + dto : dt;
    for (long long i = 0; i < nf * field; ++i) {
      const double z[2] = {(double)f[i].re, (double)f[i].im};
      fwrite(z, sizeof(double), 2, out);
    }
  }
}
int main(int argc, char** argv) {
  FILE* in = fopen(argv[1], "rb");
  FILE* out = fopen(argv[2], "wb");
  if (!in || !out) return 2;
  int hd[6];
  double sc[3];
  if (fread(hd, sizeof(int), 6, in) != 6 || fread(sc, sizeof(double), 3, in) != 3) return 3;
  std::vector<double> dts(hd[3]);
  if (fread(dts.data(), sizeof(double), dts.size(), in) != dts.size()) return 4;
  const int nf = hd[4] ? 4 : 3;
  const long long field = (long long)hd[2] * hd[1] * (hd[0] / 2 + 1);
  std::vector<double> in0(2 * nf * field), ws((size_t)hd[3] * 2 * nf * field);
  if (fread(in0.data(), sizeof(double), in0.size(), in) != in0.size()) return 5;
  if (fread(ws.data(), sizeof(double), ws.size(), in) != ws.size()) return 6;
  run<double>(hd, sc, dts, in0, ws, out);
  run<float>(hd, sc, dts, in0, ws, out);
  fclose(out);
  return 0;
}
"""


def _run_ab2v_program(tmp_path, n, dts, header_d, hist, start, per_pass):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "ab2v.cu"
    src.write_text(AB2V_PROGRAM)
    exe = tmp_path / "ab2v"
    cmd = [nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", CSRC, str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    nf = len(start)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        f.write(np.array([n, n, n, len(dts), 1 if nf == 4 else 0, hist], np.int32).tobytes())
        f.write(np.array(header_d, np.float64).tobytes())
        f.write(np.array(dts, np.float64).tobytes())
        f.write(np.ascontiguousarray(np.stack(start), np.complex128).tobytes())
        for fields in per_pass:
            f.write(np.ascontiguousarray(np.stack(fields), np.complex128).tobytes())
    r = subprocess.run([str(exe), str(fin), str(fout)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-500:]
    return np.fromfile(fout, np.complex128).reshape(2, len(dts), nf, n, n, n // 2 + 1)


def test_variable_step_ab2_update_matches_oracle(tmp_path):
    """The per-mode variable-step IF-AB2 update that ab2v_update_kernel runs
    (ab2v_point and ab2v_weights, sc_ab2v.cuh), compiled for the host,
    reproduces the oracle's passes of spectral_dns.f90:210-290 on an uneven
    step sequence when fed the oracle's right-hand sides: FP64 to 1e-13,
    FP32 to 1e-5."""
    from oracle import spectral_ref as R
    from _util import rel_l2, solenoidal_init
    n = 16
    dts = [2e-3, 2.6e-3, 1.4e-3, 2.2e-3, 1.8e-3]
    g = R.Grid(R.Params(nx=n, nu=0.01, forced=True, eps=0.1, kcut=n // 2))
    v0 = solenoidal_init(n)
    trace = []
    R.ab2v_run(v0, g, dts, trace=trace)
    out = _run_ab2v_program(tmp_path, n, dts, [g.p.nu, g.p.kcut ** 2, 1.0], 0, list(v0),
                            [list(w) for w, _ in trace])
    for p, (_, vref) in enumerate(trace):
        assert rel_l2(list(out[0, p]), list(vref)) < 1e-13, p
        assert rel_l2(list(out[1, p]), list(vref)) < 1e-5, p


@pytest.mark.parametrize("history", ["as_written", "rhs"])
def test_variable_step_scalar_update_matches_oracle(tmp_path, history):
    """The same with the passive scalar of spectral_dns_scalar.f90
    (ab2v_scalar_point, both scalar histories; velocity not truncated)."""
    from oracle import spectral_ref as R
    from _util import hermitian_fields, rel_l2, solenoidal_init
    n = 16
    dts = [2e-3, 2.6e-3, 1.4e-3, 2.2e-3, 1.8e-3]
    g = R.Grid(R.Params(nx=n, nu=0.01, forced=True, eps=0.1))
    v0 = solenoidal_init(n)
    phi0 = R.symmetrize3d(hermitian_fields((n, n, n), 7, ncomp=1)[0])
    trace = []
    R.ab2v_scalar_run(v0, phi0, g, dts, 0.7, True, 0.3, history=history, trace=trace)
    out = _run_ab2v_program(tmp_path, n, dts, [g.p.nu, 0.0, 0.7], 1 if history == "rhs" else 0,
                            list(v0) + [phi0], [list(w) + [wphi] for w, wphi, _, _ in trace])
    for p, (_, _, vref, pref) in enumerate(trace):
        assert rel_l2(list(out[0, p, :3]), list(vref)) < 1e-13, p
        assert rel_l2(out[0, p, 3], pref) < 1e-13, p
        assert rel_l2(list(out[1, p, :3]), list(vref)) < 1e-5, p
        assert rel_l2(out[1, p, 3], pref) < 1e-5, p
