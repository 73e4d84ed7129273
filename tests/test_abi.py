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
    assert "convec_dns_" in declared and "hermitianize_" in declared and len(declared) == 17
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


def _fortran_interfaces(path):
    """(function name, bind name, dummy names) of each interface in a free-form
    Fortran module, continuation lines joined."""
    import re
    text = open(path).read()
    text = re.sub(r"&\s*\n\s*", "", text)
    out = []
    for m in re.finditer(r"function\s+(\w+)\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", text):
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        out.append((m.group(1), m.group(3), args))
    return text, out


def test_fortran_module_matches_the_c_header():
    """include/specns.f90 (the ISO_C_BINDING module for the reference's
    Fortran programs) binds every function of include/specns.h under its C
    name with the C argument count, declares every dummy, and repeats the
    header's constants and the sc_params / sc_diag layouts.  No Fortran
    compiler is needed: this reads both files."""
    import re
    header = open(os.path.join(ROOT, "include", "specns.h")).read()
    decls = {m.group(1): [a for a in " ".join(m.group(2).split()).split(",") if a.strip() not in ("", "void")]
             for m in re.finditer(r"^(?:int|const char\*)\s+(sc_\w+)\(([^;]*)\);", header, re.M)}
    text, ifaces = _fortran_interfaces(os.path.join(ROOT, "include", "specns.f90"))
    assert sorted(b for _, b, _ in ifaces) == sorted(decls)
    for fname, bname, args in ifaces:
        assert fname == bname and len(args) == len(decls[bname]), bname
        body = text[text.index("function %s(" % fname):text.index("end function %s" % fname)]
        for a in args:
            assert re.search(r"::\s*%s\s*$" % a, body, re.M), (fname, a)
    for name, val in re.findall(r"^#define (SC_\w+) (\d+)", header, re.M):
        assert re.search(r"parameter :: %s = %s$" % (name, val), text, re.M), name

    def c_fields(struct):
        body = header[header.index("typedef struct %s {" % struct):]
        body = body[:body.index("}")]
        return [n for line in body.split("\n")[1:] for n in re.findall(r"(\w+)[,;]", line.split("/*")[0])]

    def f_fields(typ):
        body = text[text.index("type, bind(C) :: %s" % typ):text.index("end type %s" % typ)]
        return [n.strip() for line in body.split("\n")[1:] if "::" in line for n in line.split("::")[1].split(",")]

    for t in ("sc_params", "sc_diag"):
        assert c_fields(t) == f_fields(t), t


def test_f77_shims_report_errors_when_abort_is_off(specns_lib):
    """specns_f77_set_abort_(0): a shim given an inconsistent shape records
    SC_ERR_INVALID and returns (no abort, no CUDA call); the status is read
    once and cleared."""
    for prec in ("sp", "dp"):
        lib = _lib.load_f77(prec)
        i = ctypes.c_int
        lib.specns_f77_set_abort_(ctypes.byref(i(0)))
        st = i(-1)
        lib.specns_f77_status_(ctypes.byref(st))
        assert st.value == 0
        buf = (ctypes.c_double * 64)()
        # lx1 = 4 does not match nx = 16 (needs nx/2 + 1 = 9)
        lib.convec_dns_(buf, buf, buf, buf, buf, buf, *[ctypes.byref(i(x)) for x in (4, 16, 16, 16, 16, 16)])
        lib.specns_f77_status_(ctypes.byref(st))
        assert st.value == 1
        lib.specns_f77_status_(ctypes.byref(st))
        assert st.value == 0
        lib.specns_f77_set_abort_(ctypes.byref(i(1)))
