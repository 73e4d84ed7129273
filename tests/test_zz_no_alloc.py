"""sc_diagnostics_noalloc: diagnostics without any device allocation.

Some callers cannot call cudaMalloc -- a solver that reserves its whole
device-memory budget at start-up and must not allocate inside its step loop,
or one that cannot afford the device-wide synchronisation cudaMalloc/cudaFree
may imply.  This entry point serves them with its scratch in a static device
array.  Its results must equal those of the allocating entry point
(sc_diagnostics on a handle) on the same field, on two calls in a row (the
second call reuses the shared scratch array left by the first).  The
reductions are FP64 in both paths; tolerance 1e-12 relative.

Collected last on purpose (file name) so a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import spectral_ref as R
from _util import fresh, hermitian_fields, solenoidal_init

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.mark.parametrize("prec", [S.SC_FP64, S.SC_FP32])
def test_noalloc_diagnostics_match_handle_diagnostics(specns_lib, prec):
    torch = pytest.importorskip("torch")
    n, nu = 32, 0.01
    v = solenoidal_init(n)
    dtype = np.complex128 if prec == S.SC_FP64 else np.complex64
    v = [fresh(a, dtype) for a in v]
    with S.SpectralNS(S.default_params(n, prec, nu=nu)) as h:
        h.set_state(*v)
        d, eks = h.diagnostics()
    dev = [torch.from_numpy(a).cuda() for a in v]
    out = torch.empty(5 + n // 2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(2):
        out.fill_(float("nan"))
        rc = specns_lib.sc_diagnostics_noalloc(prec, *[C.c_void_p(t.data_ptr()) for t in dev], n, n, n,
                                               C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0, specns_lib.sc_last_error()
        stream.synchronize()
        o = out.cpu().numpy()
        assert abs(o[0] - d["energy"]) <= TOL * d["energy"]
        assert abs(2 * nu * o[1] - d["dissipation"]) <= TOL * d["dissipation"]
        assert abs(o[2] - d["max_div"]) <= TOL * max(d["max_div"], 1e-300) + 1e-300
        assert o[3] == 0 and d["nonfinite"] == 0
        assert np.max(np.abs(o[5:] - eks)) <= TOL * np.max(eks)


# Non-cubic grids, grids whose ny*nz rows do not fill one block each, and the
# grids at the scratch array's two bounds: the most shells (nx = 1024, 512
# shells) and the most blocks (ny*nz = 2^20 rows, 1024 blocks of 1024 rows).
@pytest.mark.parametrize("prec", [S.SC_FP64, S.SC_FP32])
@pytest.mark.parametrize("shape", [(64, 16, 8), (16, 16, 8), (32, 64, 64), (1024, 8, 8), (8, 1024, 1024)])
def test_noalloc_diagnostics_on_other_grids_match_oracle(specns_lib, prec, shape):
    torch = pytest.importorskip("torch")
    nx, ny, nz = shape
    v = hermitian_fields(shape, 77)
    kx, ky, kz, k2 = R.wavenumber(nx, ny, nz)
    ref = [R.energy(v), R.enstrophy(v, k2), R.max_divergence(v, kx, ky, kz)]
    ref_eks = R.spectrum(v, k2, nx)
    dtype = np.complex128 if prec == S.SC_FP64 else np.complex64
    tol = TOL if prec == S.SC_FP64 else 1e-5
    dev = [torch.from_numpy(fresh(a, dtype)).cuda() for a in v]
    out = torch.empty(5 + nx // 2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(2):
        out.fill_(float("nan"))
        rc = specns_lib.sc_diagnostics_noalloc(prec, *[C.c_void_p(t.data_ptr()) for t in dev], nx, ny, nz,
                                               C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == 0, specns_lib.sc_last_error()
        stream.synchronize()
        o = out.cpu().numpy()
        for got, want in zip(o[:3], ref):
            assert abs(got - want) <= tol * abs(want) + 1e-300
        assert o[3] == 0
        assert np.max(np.abs(o[5:] - ref_eks)) <= tol * np.max(ref_eks)


def test_noalloc_rejects_grids_beyond_its_scratch(specns_lib):
    torch = pytest.importorskip("torch")
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    rc = specns_lib.sc_diagnostics_noalloc(S.SC_FP64, p, p, p, 2048, 8, 8, p, None)
    assert rc == 1
    assert b"static scratch" in specns_lib.sc_last_error()
