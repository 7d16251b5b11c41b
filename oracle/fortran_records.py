"""Oracle (test infrastructure only): the reference's binary and XSF files,
restated in numpy to check the library's writers and readers byte for byte.

Binary files are single Fortran sequential unformatted records as gfortran
writes them with -fconvert=big-endian (Source/Makefile:86): the type-bound
write(unformatted) procedures issue child transfers that extend the parent
`write(unit) object` record (Source/density.f90:41,128-160,
Source/pot.f90:41,194-224, Source/wave.f90:37,893-921).  A record is framed
by 4-byte big-endian length markers.  Past gfortran's subrecord limit
(2**31 - 9 bytes) it is split into subrecords: a subrecord followed by
another has its leading marker negated, one that follows another its
trailing marker negated (gfortran's documented layout for long records).

XSF: Source/xsf.f90:67-128, with Fortran's F20.10, E20.10 and I5 edit
descriptors; E20.10 is rounded here from the exact binary value with
Python's decimal module (round half to even).
"""
import struct
from decimal import Decimal, ROUND_HALF_EVEN

import numpy as np

GFORTRAN_SUBRECORD = 2147483639


def record(payload: bytes, limit: int = GFORTRAN_SUBRECORD) -> bytes:
    """One sequential record around payload."""
    n = len(payload)
    if n == 0:
        return struct.pack(">i", 0) * 2
    chunks = [payload[i:i + limit] for i in range(0, n, limit)]
    out = []
    for i, c in enumerate(chunks):
        lead = -len(c) if i < len(chunks) - 1 else len(c)
        trail = -len(c) if i > 0 else len(c)
        out += [struct.pack(">i", lead), c, struct.pack(">i", trail)]
    return b"".join(out)


def read_record(data: bytes, pos: int = 0):
    """(payload, next position) of the record at pos."""
    parts, first = [], True
    while True:
        lead = struct.unpack(">i", data[pos:pos + 4])[0]
        n = abs(lead)
        parts.append(data[pos + 4:pos + 4 + n])
        trail = struct.unpack(">i", data[pos + 4 + n:pos + 8 + n])[0]
        if abs(trail) != n or (trail < 0) == first:
            raise ValueError("bad record markers")
        pos += 8 + n
        first = False
        if lead >= 0:
            return b"".join(parts), pos


def _c128(a):
    return np.asarray(a, dtype=np.complex128).ravel(order="F").astype(">c16").tobytes()


def den_payload(n_std, charge, spin=None):
    nr = np.size(charge)
    spin = np.zeros((nr, 3), dtype=np.complex128) if spin is None else spin
    return struct.pack(">3i", *n_std) + _c128(charge) + _c128(spin) + struct.pack(">i", 1)


def pot_payload(n_std, nc_pot):
    return struct.pack(">3i", *n_std) + _c128(nc_pot) + struct.pack(">i", 1)


def wvfn_payload(n_std, coeff):
    nbox, nk, nb, ns = np.shape(coeff)
    return struct.pack(">3i", *n_std) + _c128(coeff) + struct.pack(">3i", nb, nk, 1)


def parse_den(payload, nr):
    n_std = struct.unpack(">3i", payload[:12])
    a = np.frombuffer(payload[12:12 + 64 * nr], dtype=">c16").astype(np.complex128)
    alloc = struct.unpack(">i", payload[12 + 64 * nr:])[0]
    return n_std, a[:nr], a[nr:].reshape((nr, 3), order="F"), alloc


def fortran_f(x, w=20, d=10):
    """Fw.d (right-justified, d decimals, leading zero when it fits)."""
    s = f"{x:{w}.{d}f}"
    return "*" * w if len(s) > w else s


def fortran_e(x, w=20, d=10):
    """Ew.d as gfortran writes it: 0.d...d with E+ee (a three-digit exponent
    drops the E)."""
    q = Decimal(float(x))
    sign = "-" if q.is_signed() else ""           # gfortran keeps the sign of -0.0
    q = abs(q)
    if q == 0:
        digits, e = "0" * d, 0
    else:
        e = q.adjusted() + 1                      # q = 0.d1d2... x 10^e
        m = (q.scaleb(-e)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        if m >= 1:                                # rounding carried into a new digit
            e += 1
            m = (q.scaleb(-e)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        digits = str(m)[2:]
    ex = f"E{'-' if e < 0 else '+'}{abs(e):02d}" if abs(e) <= 99 else f"{'-' if e < 0 else '+'}{abs(e):03d}"
    s = f"{sign}0.{digits}{ex}"
    return s.rjust(w) if len(s) <= w else "*" * w


def xsf_text(cell, n_fine, data):
    cell = np.asarray(cell, dtype=np.float64).reshape(3, 3)
    rows = "".join(fortran_f(cell[i, 0]) + fortran_f(cell[i, 1]) + fortran_f(cell[i, 2]) + "\n"
                   for i in range(3))
    zero3 = fortran_f(0.0) * 3
    out = ["CRYSTAL\n", "PRIMVEC\n", rows, "PRIMCOORD\n", f"{1:5d}{1:5d}\n", zero3 + "\n",
           "BEGIN_BLOCK_DATAGRID_3D\n", "DATAGRID_3D_UNKNOWN\n", "BEGIN_DATAGRID_3D\n",
           "".join(f"{int(n):5d}" for n in n_fine) + "\n", zero3 + "\n", rows]
    out += [fortran_e(v) + "\n" for v in np.asarray(data, dtype=np.float64).ravel()]
    out += ["END_DATAGRID_3D\n", "END_BLOCK_DATAGRID_3D\n"]
    return "".join(out)
