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


def _expand_format(fmt):
    """Edit descriptors of a Fortran format string, repeat groups expanded:
    [('X', n) | ('A', w) | ('I', w) | ('F', w, d)]."""
    import re
    s = fmt.strip()
    assert s[0] == "(" and s[-1] == ")"
    s = s[1:-1].replace(" ", "")

    def parse(t, i):
        out = []
        while i < len(t):
            if t[i] == ",":
                i += 1
                continue
            if t[i] == ")":
                return out, i + 1
            m = re.match(r"(\d*)\(", t[i:])
            if m:
                inner, j = parse(t, i + len(m.group(0)))
                out += inner * int(m.group(1) or 1)
                i = j
                continue
            m = re.match(r"(\d+)[xX]", t[i:])
            if m:
                out.append(("X", int(m.group(1))))
                i += len(m.group(0))
                continue
            m = re.match(r"(\d*)([aAiI])(\d*)", t[i:])
            if m:
                w = int(m.group(3)) if m.group(3) else None   # A without a width: the string's length
                out += [(m.group(2).upper(), w)] * int(m.group(1) or 1)
                i += len(m.group(0))
                continue
            m = re.match(r"(\d*)[fF](\d+)\.(\d+)", t[i:])
            if m:
                out += [("F", int(m.group(2)), int(m.group(3)))] * int(m.group(1) or 1)
                i += len(m.group(0))
                continue
            raise ValueError(t[i:])
        return out, i

    return parse(s, 0)[0]


def fortran_write(fmt, *values):
    """One record of write(unit, fmt) values: X positions only when data
    follows (trailing X writes nothing), Aw right-justifies, Iw and Fw.d as
    gfortran writes them."""
    out, pending, k = "", 0, 0
    for d in _expand_format(fmt):
        if d[0] == "X":
            pending += d[1]
            continue
        if k >= len(values):
            break
        out += " " * pending
        pending = 0
        v = values[k]
        k += 1
        if d[0] == "A":
            w = len(v) if d[1] is None else d[1]
            out += v[:w] if len(v) >= w else " " * (w - len(v)) + v
        elif d[0] == "I":
            t = str(int(v))
            out += "*" * d[1] if len(t) > d[1] else t.rjust(d[1])
        else:
            out += fortran_f_edit(v, d[1], d[2])
    return out


def fortran_f_edit(x, w, d):
    """Fw.d: right-justified, w asterisks on overflow, NaN / Infinity."""
    import math
    if math.isnan(x):
        s = "NaN"
    elif math.isinf(x):
        s = "Infinity" if x > 0 else "-Infinity"
        if len(s) > w:
            s = "Inf" if x > 0 else "-Inf"
    else:
        s = f"{x:.{d}f}"
    return "*" * w if len(s) > w else s.rjust(w)


def _table_lines(kind, n_fine):
    # the library's own two comment lines stand in for io_out_file_header's
    # banner; then density_writef / pot_writef's list-directed and format-10
    # records (Source/density.f90:187-193, Source/pot.f90:252-266)
    lines = [f" # DEReK-GB300 {kind} FILE", " # values in atomic units", " " + " FFT FINE BASIS GRID  "]
    for ax, n in zip(("nx:", "ny:", "nz:"), n_fine):
        lines.append(fortran_write("(2x,a,1x,i6)", ax, n))
    lines.append("")
    return lines


def fden_text(n_fine, charge, spin=None):
    """density_writef (Source/density.f90:185-208): formats 20 and 21."""
    nr = int(np.prod(n_fine))
    spin = np.zeros((3, nr)) if spin is None else np.asarray(spin).reshape(3, nr)
    lines = _table_lines("DENSITY", n_fine)
    lines.append(fortran_write("(1x,3(a4,2x), 5x, 4(3x, A6, 1x))", "ix", "iy", "iz", "Charge", "Sx", "Sy", "Sz"))
    lines.append(" " + "-" * 65)
    n = 0
    for ix in range(1, n_fine[0] + 1):
        for iy in range(1, n_fine[1] + 1):
            for iz in range(1, n_fine[2] + 1):
                lines.append(fortran_write("(1x,3(i4,2x), 5x, 4(f9.4,2x))", ix, iy, iz, float(charge[n]),
                                           float(spin[0, n]), float(spin[1, n]), float(spin[2, n])))
                n += 1
    return "\n".join(lines) + "\n"


def fpot_text(n_fine, nc_pot):
    """pot_writef (Source/pot.f90:250-284): formats 20 and 21, columns
    (1,1), (1,2), (2,1), (2,2) as real and imaginary parts."""
    nc = np.asarray(nc_pot, dtype=np.complex128).reshape(-1, 2, 2)
    lines = _table_lines("POTENTIAL", n_fine)
    lines.append(fortran_write("(1x,3(a4,2x), 5x, 4(9x, A5, 6x, 4x))", "ix", "iy", "iz",
                               "(1,1)", "(1,2)", "(2,1)", "(2,2)"))
    lines.append(" " + "-" * 115)
    n = 0
    for ix in range(1, n_fine[0] + 1):
        for iy in range(1, n_fine[1] + 1):
            for iz in range(1, n_fine[2] + 1):
                v = []
                for i, j in ((0, 0), (0, 1), (1, 0), (1, 1)):
                    v += [float(nc[n, i, j].real), float(nc[n, i, j].imag)]
                lines.append(fortran_write("(1x,3(i4,2x), 5x, 4(f9.4,2x,f9.4,4x))", ix, iy, iz, *v))
                n += 1
    return "\n".join(lines) + "\n"
