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
