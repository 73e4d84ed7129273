"""The C-ABI library loads and exports every symbol its headers declare (no GPU)."""
import ctypes
import glob
import os

from speccodelib_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(specns_lib):
    declared = _lib.declared_symbols(os.path.join(ROOT, "include", "specns.h"))
    assert len(declared) >= 20
    missing = [n for n in declared if not hasattr(specns_lib, n)]
    assert missing == []


def test_every_declared_symbol_has_a_binding():
    declared = _lib.declared_symbols(os.path.join(ROOT, "include", "specns.h"))
    assert sorted(declared) == sorted(_lib.SIGNATURES)


def test_default_params_and_errors_without_gpu(specns_lib):
    import speccodelib_gb300 as s
    p = s.default_params(64, s.SC_FP64)
    assert (p.nx, p.ny, p.nz) == (64, 64, 64)
    assert p.nu == 0.01 and p.dt == 2e-3 and p.eps == 0.1 and p.fkmax == 2.5
    bad = s.default_params(48)          # not a power of two -> SC_ERR_INVALID before any CUDA call
    h = ctypes.c_void_p()
    rc = specns_lib.sc_create(ctypes.byref(bad), ctypes.byref(h))
    assert rc == 1 and b"power of two" in specns_lib.sc_last_error()
    assert not h.value


def test_f77_shims_export_every_declared_symbol(specns_lib):
    declared = _lib.declared_f77_symbols()
    assert "convec_dns_" in declared and "hermitianize_" in declared and len(declared) == 15
    for prec in ("sp", "dp"):
        lib = _lib.load_f77(prec)
        missing = [n for n in declared if not hasattr(lib, n)]
        assert missing == [], (prec, missing)


def test_rot_steps_rejects_bad_arguments_without_gpu(specns_lib):
    """sc_rot_steps checks its handle and arguments before any CUDA call."""
    assert specns_lib.sc_rot_steps(None, 1, 1.0, 0.0, 2.5) == 1    # SC_ERR_INVALID
    assert specns_lib.sc_rot_steps(None, -1, 1.0, 0.0, 2.5) == 1


def test_ab2v_step_rule_matches_oracle(specns_lib):
    """sc_ab2v_dt (host code, no GPU) is the oracle's step rule of
    spectral_dns.f90:212-217 on a sweep that crosses all three branches, and
    the variable-step entry points reject bad arguments before any CUDA call."""
    import numpy as np
    import speccodelib_gb300 as s
    from oracle import spectral_ref as R
    rng = np.random.default_rng(3)
    for _ in range(2000):
        betadx, umax = rng.uniform(0.01, 0.5), rng.uniform(0.5, 5.0)
        dto, time = rng.uniform(1e-3, 0.2), rng.uniform(0.0, 1.0)
        twrite = time + rng.uniform(1e-4, 0.3)
        assert s.ab2v_dt(betadx, umax, dto, time, twrite) == R.ab2v_dt(betadx, umax, dto, time, twrite)
    d = ctypes.c_double()
    assert specns_lib.sc_ab2v_dt(0.1, 0.0, 1.0, 0.0, 1.0, ctypes.byref(d)) == 1
    assert specns_lib.sc_ab2v_pass(None, 1e-3) == 1
    p = ctypes.c_int()
    assert specns_lib.sc_ab2v_state(None, ctypes.byref(p), ctypes.byref(d)) == 1


def test_scalar_entry_points_reject_bad_arguments_without_gpu(specns_lib):
    assert specns_lib.sc_set_scalar(None, None) == 1
    assert specns_lib.sc_get_scalar(None, None) == 1
    assert specns_lib.sc_rot_scalar_steps(None, 1, 1.0, 0.0, 2.5, 1.0, 0, 0.0) == 1


def test_scalar_file_entry_points_reject_bad_arguments_without_gpu(specns_lib):
    assert specns_lib.sc_outputphi(None, b".", 0, 0) == 1
    assert specns_lib.sc_inputphi(None, b".", 0, 0) == 1


def test_ab2v_scalar_pass_rejects_bad_arguments_without_gpu(specns_lib):
    assert specns_lib.sc_ab2v_scalar_pass(None, 1e-3, 1.0, 0, 0.0, 0) == 1
