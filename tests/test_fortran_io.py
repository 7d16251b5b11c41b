"""The reference's binary and XSF files: the library's writers and readers
against the oracle's restatement of the gfortran record layout, byte for
byte (host only, no GPU)."""
import os

import numpy as np
import pytest

from oracle import fortran_records as F


@pytest.fixture(autouse=True)
def _default_subrecords():
    import derek_gb300 as dg
    dg.set_subrecord_limit(0)
    yield
    dg.set_subrecord_limit(0)


def _rand_c(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _read(path):
    with open(path, "rb") as f:
        return f.read()


def test_den_bytes_and_round_trip(tmp_path):
    import derek_gb300 as dg
    rng = np.random.default_rng(1)
    nr, ns = 7 * 5 * 3, (4, 3, 2)
    charge = _rand_c(rng, nr)
    spin = np.asfortranarray(_rand_c(rng, (nr, 3)))
    p = tmp_path / "a.den"
    dg.write_den(p, ns, charge, spin)
    assert _read(p) == F.record(F.den_payload(ns, charge, spin))
    c2, s2 = dg.read_den(p, ns, nr)
    assert np.array_equal(c2, charge) and np.array_equal(s2, spin)
    # no spin: the reference's zero spin density
    dg.write_den(p, ns, charge.real.astype(np.complex128))
    n_std, c3, s3, alloc = F.parse_den(F.read_record(_read(p))[0], nr)
    assert n_std == ns and alloc == 1 and np.array_equal(c3, charge.real) and not s3.any()


def test_pot_and_wvfn_bytes(tmp_path):
    import derek_gb300 as dg
    rng = np.random.default_rng(2)
    nr, ns = 60, (3, 3, 3)
    nc = np.asfortranarray(_rand_c(rng, (nr, 2, 2)))
    p = tmp_path / "a.pot"
    dg.write_pot(p, ns, nc)
    assert _read(p) == F.record(F.pot_payload(ns, nc))
    assert np.array_equal(dg.read_pot(p, ns, nr), nc)
    coeff = np.asfortranarray(_rand_c(rng, (27, 2, 3, 2)))
    w = tmp_path / "a.wvfn"
    dg.write_wvfn(w, ns, coeff)
    assert _read(w) == F.record(F.wvfn_payload(ns, coeff))
    assert np.array_equal(dg.read_wvfn(w, ns, 27, 2, 3, 2), coeff)


@pytest.mark.parametrize("limit", [100, 64, 17])
def test_subrecords(tmp_path, limit):
    """Records past the subrecord limit split with negated continuation
    markers (exercised with a small limit; gfortran's is 2**31 - 9)."""
    import derek_gb300 as dg
    rng = np.random.default_rng(3)
    nr, ns = 10, (2, 2, 2)
    charge = _rand_c(rng, nr)
    dg.set_subrecord_limit(limit)
    p = tmp_path / "s.den"
    dg.write_den(p, ns, charge)
    data = _read(p)
    assert data == F.record(F.den_payload(ns, charge), limit)
    assert F.read_record(data)[0] == F.den_payload(ns, charge)
    c2, _ = dg.read_den(p, ns, nr)
    assert np.array_equal(c2, charge)


def test_readers_reject_bad_files(tmp_path):
    import derek_gb300 as dg
    rng = np.random.default_rng(4)
    nr, ns = 8, (2, 2, 2)
    nc = _rand_c(rng, (nr, 2, 2))
    p = tmp_path / "b.pot"
    dg.write_pot(p, ns, nc)
    with pytest.raises(dg.DerekError):   # standard grid mismatch (Source/pot.f90:329-331)
        dg.read_pot(p, (2, 2, 3), nr)
    with pytest.raises(dg.DerekError):   # wrong size
        dg.read_pot(p, ns, nr + 1)
    data = _read(p)
    q = tmp_path / "t.pot"
    q.write_bytes(data[:-6])
    with pytest.raises(dg.DerekError):   # truncated
        dg.read_pot(q, ns, nr)
    q.write_bytes(data[:-4] + (12345).to_bytes(4, "big"))
    with pytest.raises(dg.DerekError):   # trailing marker does not match
        dg.read_pot(q, ns, nr)


def test_fortran_e_known_answers():
    assert F.fortran_e(1.5) == "    0.1500000000E+01"
    assert F.fortran_e(-0.000123) == "   -0.1230000000E-03"
    assert F.fortran_e(0.0) == "    0.0000000000E+00"
    assert F.fortran_e(1e-100) == "    0.1000000000E-99"
    assert F.fortran_e(1e-101) == "    0.1000000000-100"
    assert F.fortran_e(1e101) == "    0.1000000000+102"
    assert F.fortran_f(-2.5) == "       -2.5000000000"


def test_xsf_matches_oracle(tmp_path):
    import derek_gb300 as dg
    rng = np.random.default_rng(5)
    n = (3, 4, 2)
    data = rng.standard_normal(24) * 10.0 ** rng.integers(-120, 120, 24)
    data[:6] = [0.0, -0.0, 0.99999999995, -1.5, 123456.789, 1e-100]
    cell = np.array([[10.0, 0.1, 0.0], [0.0, 9.5, -0.25], [0.3, 0.0, 11.0]])
    p = tmp_path / "v.xsf"
    dg.write_xsf(p, cell, n, data)
    assert p.read_text() == F.xsf_text(cell, n, data)


def test_formatted_tables_match_oracle(tmp_path):
    """.fden / .fpot tables byte for byte against the oracle, which applies
    the reference's own format strings through an edit-descriptor
    interpreter (overflow, negative zero, NaN included)."""
    import derek_gb300 as dg
    rng = np.random.default_rng(5)
    n = (3, 4, 2)
    nr = int(np.prod(n))
    charge = rng.uniform(0, 2, nr)
    charge[0], charge[1], charge[2] = 12345.6789, -0.00004, float("nan")
    spin = rng.standard_normal((3, nr))
    p = tmp_path / "a.fden"
    dg.write_fden(p, n, charge, spin)
    assert p.read_text() == F.fden_text(n, charge, spin)
    dg.write_fden(p, n, charge)
    assert p.read_text() == F.fden_text(n, charge)
    nc = rng.standard_normal((nr, 2, 2)) + 1j * rng.standard_normal((nr, 2, 2))
    nc[3, 0, 1] = -1e9
    q = tmp_path / "a.fpot"
    dg.write_fpot(q, n, nc)
    assert q.read_text() == F.fpot_text(n, nc)
    rows = q.read_text().splitlines()
    assert rows[7].startswith("   ix    iy    iz                (1,1)") and set(rows[8]) == {" ", "-"}
