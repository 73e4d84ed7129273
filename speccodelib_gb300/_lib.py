"""Loader for the in-tree CUDA library ``lib/libspecns.so`` (ctypes).

The library is built in place by ``speccodelib_gb300.build``.  Loading it
needs no GPU; calling a compute entry point does.  There is no fallback: if
the library is missing, `load()` raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libspecns.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "specns.h")

_LIB = None

_P = C.c_void_p
_I = C.c_int
_D = C.c_double
_LL = C.c_longlong
_CS = C.c_char_p

# argument types of every function declared in include/specns.h
SIGNATURES = {
    "sc_last_error": ([], C.c_char_p),
    "sc_default_params": ([_P, _I, _I], _I),
    "sc_create": ([_P, _P], _I),
    "sc_destroy": ([_P], _I),
    "sc_set_device": ([_I], _I),
    "sc_set_stream": ([_P, _P], _I),
    "sc_set_dt": ([_P, _D], _I),
    "sc_set_state": ([_P, _P, _P, _P], _I),
    "sc_get_state": ([_P, _P, _P, _P], _I),
    "sc_set_state_device": ([_P, _P, _P, _P], _I),
    "sc_get_state_device": ([_P, _P, _P, _P], _I),
    "sc_init_field": ([_P, _I, _I, _D, _D, _D, _D], _I),
    "sc_rhs": ([_P, _P, _P, _P], _I),
    "sc_rk4_steps": ([_P, _I], _I),
    "sc_ab2_steps": ([_P, _I], _I),
    "sc_rot_steps": ([_P, _I, _D, _D, _D], _I),
    "sc_outputphi": ([_P, _CS, _I, _I], _I),
    "sc_inputphi": ([_P, _CS, _I, _I], _I),
    "sc_hermitianize": ([_I, _P, _I, _I, _I], _I),
    "sc_forcephi": ([_I, _P, _P, _I, _I, _I, _D, _D], _I),
    "sc_forcephi_rot": ([_I, _P, _P, _I, _I, _I, _D, _D, _D], _I),
    "sc_set_scalar": ([_P, _P], _I),
    "sc_get_scalar": ([_P, _P], _I),
    "sc_rot_scalar_steps": ([_P, _I, _D, _D, _D, _D, _I, _D], _I),
    "sc_ab2v_pass": ([_P, _D], _I),
    "sc_ab2v_scalar_pass": ([_P, _D, _D, _I, _D, _I], _I),
    "sc_ab2v_state": ([_P, C.POINTER(_I), C.POINTER(_D)], _I),
    "sc_ab2v_dt": ([_D, _D, _D, _D, _D, C.POINTER(_D)], _I),
    "sc_diagnostics": ([_P, _P, _P], _I),
    "sc_get_params": ([_P, _P], _I),
    "sc_output3d": ([_P, _CS, _I, _I], _I),
    "sc_input3d": ([_P, _CS, _I, _I], _I),
    "sc_fortran_record_write": ([_CS, _P, _LL, _LL], _I),
    "sc_fortran_record_read": ([_CS, _P, _LL], _I),
    "sc_adjoint_rk4": ([_P, _I, _I, _I, _I, _P, _P, _P, _P], _I),
    "sc_adjoint_rk4_vjp": ([_P, _I, _I, _P, _P, _P, _P, _P, _P], _I),
    "sc_set_adjoint_budget": ([_P, _D], _I),
    "sc_adjoint_kept_segments": ([_P, _P], _I),
    "sc_profile_enable": ([_P, _I], _I),
    "sc_profile_read": ([_P, C.c_char_p, _P, _P], _I),
    "sc_fp64_peak_probe": ([_P], _I),
    "sc_step_bytes": ([_P, _P], _I),
    "sc_diagnostics_noalloc": ([_I, _P, _P, _P, _I, _I, _I, _P, _P], _I),
    "sc_ens_create": ([_I, _I, _P, _P, _P, _D, _P], _I),
    "sc_ens_destroy": ([_P], _I),
    "sc_ens_set_stream": ([_P, _P], _I),
    "sc_ens_set_member": ([_P, _I, _P], _I),
    "sc_ens_get_member": ([_P, _I, _P], _I),
    "sc_ens_init": ([_P, _P, _D, _D], _I),
    "sc_ens_rk4_steps": ([_P, _I, _I], _I),
    "sc_ens_uses_graph": ([_P], _I),
    "sc_ens_tune": ([_P, _I, _P], _I),
    "sc_ens_set_variant": ([_P, _I], _I),
    "sc_ens_variant": ([_P, _P, _P, _P, _P], _I),
    "sc_convec_dns": ([_I, _P, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I], _I),
    "sc_projection": ([_I, _P, _P, _P, _I, _I, _I], _I),
    "sc_force": ([_I, _P, _P, _P, _P, _P, _P, _I, _I, _I, _D, _D], _I),
    "sc_force_rot": ([_I, _P, _P, _P, _P, _P, _P, _I, _I, _I, _D, _D, _D], _I),
    "sc_convecphi_dns": ([_I, _P, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I], _I),
    "sc_skewness": ([_I, _P, _I, _I, _I, _P], _I),
    "sc_enstrophy": ([_I, _P, _P, _P, _P, _I, _I, _I, _I, _I, _I], _I),
    "sc_symmetrize": ([_I, _P, _I, _I, _I], _I),
    "sc_dealiasing": ([_I, _P, _I, _I, _I], _I),
    "sc_smag": ([_I, _P, _P, _P] + [_P] * 6 + [_I] * 6 + [_D, _D], _I),
    "sc_dynsmag": ([_I, _P, _P, _P] + [_P] * 6 + [_I] * 6 + [_D, _D, _D, _P, _P, _P, _I], _I),
}


def declared_symbols(header=HEADER):
    """Names of the functions declared in a C header of include/."""
    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sc_[a-z0-9_]+)\s*\(", src)))


F77_HEADER = os.path.join(os.path.dirname(HERE), "include", "specns_f77.h")
F77_LIBS = {"sp": os.path.join(HERE, "lib", "libspecns_f77_sp.so"),
            "dp": os.path.join(HERE, "lib", "libspecns_f77_dp.so")}


def declared_f77_symbols(header=F77_HEADER):
    """Fortran entry points declared in include/specns_f77.h."""
    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\bvoid\s+([A-Za-z0-9_]+)\s*\(", src)))


def load_f77(prec="dp"):
    """Load a Fortran-ABI shim library ('sp' or 'dp'); needs libspecns.so beside it."""
    load()
    return C.CDLL(F77_LIBS[prec])


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise OSError("libspecns.so is not built (%s); run speccodelib_gb300.build.build()" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _LIB = lib
    return lib
