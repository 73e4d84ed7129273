"""Fortran unformatted records (the reference's output3d / input3d files):
the library's host-side writer and reader against the restated gfortran
format (oracle/fortran_record.py), including subrecord splitting; no GPU."""
import ctypes as C

import numpy as np
import pytest

from oracle import fortran_record as FR
from speccodelib_gb300 import _lib


@pytest.fixture(scope="module")
def lib():
    from speccodelib_gb300 import build
    build.build()
    return _lib.load()


@pytest.mark.parametrize("nbytes,max_sub", [(0, 0), (48, 0), (2500, 1000), (3000, 1000), (7, 3)])
def test_record_bytes_match_gfortran_layout(lib, tmp_path, nbytes, max_sub):
    data = np.random.default_rng(nbytes).integers(0, 256, nbytes, dtype=np.uint8).tobytes()
    path = str(tmp_path / "r.dat").encode()
    buf = C.create_string_buffer(data, max(nbytes, 1))
    assert lib.sc_fortran_record_write(path, buf, nbytes, max_sub) == 0
    raw = open(path, "rb").read()
    assert raw == FR.record_bytes(data, max_sub if max_sub else FR.MAX_SUBRECORD)
    assert FR.read_record(raw) == data
    back = C.create_string_buffer(max(nbytes, 1))
    assert lib.sc_fortran_record_read(path, back, nbytes) == 0
    assert back.raw[:nbytes] == data


def test_record_reader_rejects_mismatches(lib, tmp_path):
    path = str(tmp_path / "r.dat").encode()
    data = bytes(range(64))
    open(path, "wb").write(FR.record_bytes(data, 20))
    back = C.create_string_buffer(64)
    assert lib.sc_fortran_record_read(path, back, 64) == 0 and back.raw == data
    assert lib.sc_fortran_record_read(path, back, 63) != 0      # longer than expected
    big = C.create_string_buffer(80)
    assert lib.sc_fortran_record_read(path, big, 80) != 0       # shorter than expected
    open(path, "wb").write(FR.record_bytes(data)[:-2])
    assert lib.sc_fortran_record_read(path, back, 64) != 0      # truncated
    assert lib.sc_fortran_record_read(str(tmp_path / "none.dat").encode(), back, 64) != 0
