"""Restatement of the gfortran sequential unformatted record format (test
infrastructure: the oracle for sc_fortran_record_write / sc_output3d).

The reference writes its fields with `write(10) ux` on a unit opened
`form='unformatted'` (output.f90:103-132) and reads them back with
`read(10) ux` (input.f90:106-136).  The byte format is gfortran's, a
third-party dependency whose version the reference does not pin; its
documented layout: a record is one or more subrecords, each a 4-byte
little-endian signed length marker, the data, and the marker again; at most
2147483639 data bytes per subrecord; a leading marker is negative when more
subrecords follow, a trailing marker negative when a subrecord precedes.
"""
import struct

MAX_SUBRECORD = 2147483639


def record_bytes(data: bytes, max_sub: int = MAX_SUBRECORD) -> bytes:
    out = []
    pos, first = 0, True
    while True:
        chunk = data[pos:pos + max_sub]
        pos += len(chunk)
        more = pos < len(data)
        out.append(struct.pack("<i", -len(chunk) if more else len(chunk)))
        out.append(chunk)
        out.append(struct.pack("<i", len(chunk) if first else -len(chunk)))
        first = False
        if not more:
            return b"".join(out)


def read_record(buf: bytes) -> bytes:
    data, pos, first = [], 0, True
    while True:
        (lead,) = struct.unpack_from("<i", buf, pos)
        n = abs(lead)
        data.append(buf[pos + 4:pos + 4 + n])
        (trail,) = struct.unpack_from("<i", buf, pos + 4 + n)
        assert abs(trail) == n and (trail < 0) != first
        pos += 8 + n
        first = False
        if lead >= 0:
            return b"".join(data)
