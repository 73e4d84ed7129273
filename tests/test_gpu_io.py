"""sc_output3d / sc_input3d: the state as the reference's output3d writes it
(u{x,y,z}<n>.dat, one Fortran unformatted record of complex(sp)
(nx/2+1, ny, nz) each) and back."""
import os

import numpy as np
import pytest

import speccodelib_gb300 as S
from oracle import fortran_record as FR
from _util import rel_l2, solenoidal_init

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [S.SC_FP64, S.SC_FP32])
def test_output3d_files_and_round_trip(specns_lib, prec, tmp_path):
    n = 32
    v = solenoidal_init(n)
    dt = np.complex128 if prec == S.SC_FP64 else np.complex64
    with S.SpectralNS(S.default_params(n, prec)) as h:
        h.set_state(*v)
        h.rk4_steps(2)
        state = h.get_state()
        h.output3d(tmp_path, 7)
        for c, name in enumerate(("ux", "uy", "uz")):
            raw = open(os.path.join(tmp_path, "%s7.dat" % name), "rb").read()
            arr = np.frombuffer(FR.read_record(raw), dtype=dt).reshape(state[c].shape)
            assert np.array_equal(arr, state[c])          # Fortran order == (nz, ny, nx/2+1) C order
        h.rk4_steps(1)
        h.input3d(tmp_path, 7)
        assert all(np.array_equal(a, b) for a, b in zip(h.get_state(), state))
        # a reference build of the other precision: converted on the way out and in
        other = S.SC_FP32 if prec == S.SC_FP64 else S.SC_FP64
        h.output3d(tmp_path, 8, file_precision=other)
        h.input3d(tmp_path, 8, file_precision=other)
        assert rel_l2(h.get_state(), state) < (1e-7 if prec == S.SC_FP64 else 1e-15)
        with pytest.raises(S.SpecNSError):
            h.input3d(tmp_path, 99)                        # no such files


@pytest.mark.parametrize("prec", [S.SC_FP64, S.SC_FP32])
@pytest.mark.parametrize("mode", ["direct", "staged", "strided"])
def test_state_round_trip_pinned_and_pageable(specns_lib, prec, mode, monkeypatch):
    """sc_set_state / sc_get_state through pinned (cudaHostAlloc) and pageable
    host buffers under each host copy path (SPECNS_COPY; the default reads
    and writes pinned memory from the device): the state comes back bit for
    bit, on a non-cubic grid, and a step from either kind of buffer agrees."""
    torch = pytest.importorskip("torch")
    from speccodelib_gb300 import specns as SP
    from _util import hermitian_fields
    monkeypatch.setenv("SPECNS_COPY", mode)
    nx, ny, nz = 64, 32, 16
    cdt = np.complex128 if prec == S.SC_FP64 else np.complex64
    tdt = torch.complex128 if prec == S.SC_FP64 else torch.complex64
    v = [np.ascontiguousarray(a, cdt) for a in hermitian_fields((nx, ny, nz), 91)]
    shape = v[0].shape

    def pinned():
        return torch.empty(shape, dtype=tdt, pin_memory=True).numpy()

    p = S.default_params(nx, prec, ny=ny, nz=nz)
    with S.SpectralNS(p) as h:
        src = [pinned() for _ in range(3)]
        for s_, a in zip(src, v):
            s_[...] = a
        SP._check(SP.lib().sc_set_state(h.h, *[SP._ptr(a) for a in src]))
        back = [pinned() for _ in range(3)]
        SP._check(SP.lib().sc_get_state(h.h, *[SP._ptr(a, True) for a in back]))
        for a, b in zip(back, v):
            assert np.array_equal(a, b)
        assert all(np.array_equal(a, b) for a, b in zip(h.get_state(), v))   # pageable out
        h.rk4_steps(1)
        w_pinned = h.get_state()
        h.set_state(*v)                                                       # pageable in
        h.rk4_steps(1)
        w_pageable = h.get_state()
    for a, b in zip(w_pinned, w_pageable):
        assert np.array_equal(a, b)


def test_state_round_trip_misaligned_pinned(specns_lib):
    """FP64 state from and to pinned host buffers that start 8 bytes past a
    16-byte boundary (complex128 elements the repack kernel cannot move whole):
    the copy takes the staged path and the state comes back bit for bit."""
    torch = pytest.importorskip("torch")
    from speccodelib_gb300 import specns as SP
    from _util import hermitian_fields
    import ctypes as C
    nx, ny, nz = 32, 16, 8
    v = [np.ascontiguousarray(a, np.complex128) for a in hermitian_fields((nx, ny, nz), 93)]
    nbytes = v[0].nbytes
    bufs = [torch.empty(nbytes + 16, dtype=torch.uint8, pin_memory=True) for _ in range(6)]
    ptrs = [b.data_ptr() + (8 if b.data_ptr() % 16 == 0 else 0) for b in bufs]
    assert all(p % 16 == 8 for p in ptrs)
    for p_, a in zip(ptrs[:3], v):
        C.memmove(p_, a.ctypes.data, nbytes)
    p = S.default_params(nx, S.SC_FP64, ny=ny, nz=nz)
    with S.SpectralNS(p) as h:
        SP._check(SP.lib().sc_set_state(h.h, *[C.c_void_p(x) for x in ptrs[:3]]))
        SP._check(SP.lib().sc_get_state(h.h, *[C.c_void_p(x) for x in ptrs[3:]]))
    for p_, a in zip(ptrs[3:], v):
        out = np.empty_like(a)
        C.memmove(out.ctypes.data, p_, nbytes)
        assert np.array_equal(out, a)
