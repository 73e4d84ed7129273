"""Build recipe for the CUDA library (sm_103a only).

Compiles every ``csrc/*.cu`` translation unit in parallel with nvcc and links
``libspecns.so`` in place (next to this file, under ``lib/``).  The f77-style
shim libraries (``libspecns_f77_sp.so`` / ``libspecns_f77_dp.so``, the
reference's Fortran entry points ``convec_dns_`` etc.) are linked from
``csrc/f77/sc_f77.cpp`` against the main library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libspecns.so")
F77_SRC = os.path.join(CSRC, "f77", "sc_f77.cpp")
F77_LIBS = {"sp": os.path.join(LIBDIR, "libspecns_f77_sp.so"),
            "dp": os.path.join(LIBDIR, "libspecns_f77_dp.so")}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "--expt-relaxed-constexpr"]
# Extra preprocessor definitions for tuning builds, e.g.
# SPECNS_NVCC_DEFINES="SC_NO_F32X2 ZI_DIV=8"; a change rebuilds every object.
DEFINES = ["-D" + d for d in os.environ.get("SPECNS_NVCC_DEFINES", "").split()]
STAMP = os.path.join(BUILD, "defines.txt")


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build")
    return cand


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "specns.h"))
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, verbose):
    obj = os.path.join(BUILD, src[:-3] + ".o")
    deps = [os.path.join(CSRC, src)] + _headers()
    if not _stale(obj, deps):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *DEFINES, "-c", os.path.join(CSRC, src), "-o", obj + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-4000:]))
    if verbose and r.stderr.strip():
        print(r.stderr[-2000:], file=sys.stderr)
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose=False, jobs=None):
    """Compile (incrementally) and link; returns the path of libspecns.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    stamp = " ".join(DEFINES)
    old = open(STAMP).read() if os.path.exists(STAMP) else ""
    if old != stamp:
        for f in os.listdir(BUILD):
            if f.endswith(".o"):
                os.remove(os.path.join(BUILD, f))
        with open(STAMP, "w") as fh:
            fh.write(stamp)
    srcs = _sources()
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if _stale(LIB, objs):
        tmp = LIB + ".%d.tmp" % os.getpid()
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s" % r.stderr[-4000:])
        os.replace(tmp, LIB)
    if os.path.exists(F77_SRC):
        for prec, out in F77_LIBS.items():
            if _stale(out, [F77_SRC, LIB] + _headers()):
                tmp = out + ".%d.tmp" % os.getpid()
                cmd = ["g++", "-O2", "-fPIC", "-shared", "-std=c++17",
                       "-DSC_F77_%s" % prec.upper(),
                       "-I", os.path.join(os.path.dirname(HERE), "include"),
                       F77_SRC, "-o", tmp, "-L", LIBDIR, "-lspecns",
                       "-Wl,-rpath,$ORIGIN"]
                r = subprocess.run(cmd, capture_output=True, text=True)
                if r.returncode != 0:
                    raise RuntimeError("f77 shim build failed:\n%s" % r.stderr[-4000:])
                os.replace(tmp, out)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
