"""The .info reader (derek_info_read) against the oracle's restatement of
Source/io.f90's reader, and the unit constants against CODATA 2018
(host only, no GPU)."""
import numpy as np
import pytest

from oracle import info_reader as O

LATTICE = "$DATA LATTICE\n5.0 0.0 0.0\n0.0 5.5 0.1\n0.0 0.0 6.0\n$ENDDATA LATTICE\n"

CASES = {
    "basic": "cut_off_energy : 500\nn_electrons : 8\nconduction_bands= 4\nelectronic_temp : 300\n"
             "kpt_mp_grid : 2 2 2\ntask : dos\n! a comment line\n# another\n" + LATTICE,
    "units": "unit_energy : Ry\nunit_length : nm\n" + LATTICE + "cut_off_energy : 3.5\nenergy_tol = 1.0d-5\n"
             "finite_barrier_width : 0.1 0.2 0.3\nunit_efield : Ha/Bohr/e\next_efield : 0.1 0 0\n"
             "unit_bfield : G\next_bfield : 0 0 2e4\nelectronic_temp : 1000\n",
    "units_after_block": LATTICE + "unit_length : bohr\nunit_energy : meV\ncut_off_energy : 8000\n"
                         "electronic_temp : 100\n",
    "typos": "cut_of_energy : 300\nn_electron : 4\nconduction_band : 2\nenergi_tol : 1e-6\nelectronic_temp : 50\n"
             + LATTICE,
    "list_forms": "kpt_mp_grid : 3*2\ndos_kpt_mp_grid = 4,5,6\nwrite_wvfn : .TRUE.\nsoc : F\ntask : 'bandstructure'\n"
                  "periodic_pot_grid : 1 2 / 9\nprint_level : 3\nelectronic_temp : 10\n" + LATTICE,
    "output_none": "output_level : none\nelectronic_temp : 10\n" + LATTICE,
    "output_all": "output_level : all\nelectronic_temp : 10\n" + LATTICE,
    "gaussian": "unit_energy : Ha\nunit_length : bohr\n$DATA GAUSSIAN_POT\n0.1 0.2 0.3 1.5 0.9\n"
                "# skipped\n  0.9 0.9 0.9 9.0 9.0\n0.5 0.5 0.5 2.0 1.2\n$ENDDATA GAUSSIAN_POT\n"
                "electronic_temp : 10\n" + LATTICE,
    # the key field runs to column 40; the number starts at column 56 and the 60-column cut keeps 12345
    "truncation": "cut_off_energy" + " " * 26 + ":" + " " * 14 + "123456789\n"
                  "electronic_temp : 10\n" + LATTICE,
    "comment_bang": "cut_off_energy : 100 ! not read\nelectronic_temp : 10\n" + LATTICE,
}

ERRORS = {
    "unknown_key": "blahblah : 1\n" + LATTICE,
    "duplicate": "max_scf : 4\nmax_scf : 5\n" + LATTICE,
    "no_lattice": "max_scf : 4\n",
    "lattice_rows": "$DATA LATTICE\n5 0 0\n  0 5 0\n0 0 5\n$ENDDATA LATTICE\n",   # an indented row is a comment
    "unknown_block": "$DATA FOO\n1 2 3\n$ENDDATA FOO\n" + LATTICE,
    "bad_task": "task : relax\n" + LATTICE,
    "print_level": "print_level : 5\n" + LATTICE,
    "gaussian_key": "external_pot : gaussian_pot\n" + LATTICE,
    "bad_value": "max_scf : 4.5\n" + LATTICE,
    "no_separator": "max_scf 4\n" + LATTICE,
    "lattice_key": "lattice : 3\n" + LATTICE,
    "unit": "unit_energy : furlong\n" + LATTICE,
    "short_list": "kpt_mp_grid : 2 2\n" + LATTICE,   # fewer values than the array and no '/' 
}


def _lib_read(tmp_path, text):
    import derek_gb300 as dg
    p = tmp_path / "case.info"
    p.write_text(text)
    return dg.read_info(p), p


@pytest.mark.parametrize("name", sorted(CASES))
def test_info_matches_oracle(tmp_path, name):
    got, path = _lib_read(tmp_path, CASES[name])
    ref = O.read_info(path)
    for k, v in ref.items():
        if k in ("corrected", "pot_centres", "pot_heights", "pot_widths"):
            continue
        g = got[k]
        if isinstance(v, list):
            assert list(g[:len(v)]) == v, (k, g, v)
        else:
            assert g == v, (k, g, v)
    n = ref["n_pots"]
    assert got["pot_centres"][:3 * n] == ref["pot_centres"]
    assert got["pot_heights"][:n] == ref["pot_heights"] and got["pot_widths"][:n] == ref["pot_widths"]
    assert got["n_corrected"] == len(ref["corrected"])


@pytest.mark.parametrize("name", sorted(ERRORS))
def test_info_errors(tmp_path, name):
    import derek_gb300 as dg
    p = tmp_path / "bad.info"
    p.write_text(ERRORS[name])
    with pytest.raises(O.InfoError):
        O.read_info(p)
    with pytest.raises(dg.DerekError):
        dg.read_info(p)


def test_reader_quirks(tmp_path):
    got, _ = _lib_read(tmp_path, CASES["units_after_block"])
    # the lattice was read before unit_length changed: the default angstrom applies
    assert got["cell"][0] == pytest.approx(5.0 * O.units()["A"], rel=1e-15)
    assert got["cut_off_energy"] == pytest.approx(8.0 * O.units()["eV"], rel=1e-15)   # 8000 meV
    got, _ = _lib_read(tmp_path, CASES["comment_bang"])
    assert got["cut_off_energy"] == pytest.approx(200.0 * O.units()["eV"])   # the '!' line is skipped
    got, _ = _lib_read(tmp_path, CASES["truncation"])
    assert got["cut_off_energy"] == pytest.approx(12345.0 * O.units()["eV"])   # 60-character lines
    got, _ = _lib_read(tmp_path, CASES["list_forms"])
    assert list(got["kpt_mp_grid"]) == [2, 2, 2] and list(got["dos_kpt_mp_grid"]) == [4, 5, 6]
    assert list(got["periodic_pot_grid"]) == [1, 2, 1]   # '/' ends the read; the third keeps its default
    assert got["task"] == "bandstructure" and got["write_wvfn"] == 1 and got["soc"] == 0
    got, _ = _lib_read(tmp_path, CASES["typos"])
    assert got["n_corrected"] == 4 and got["n_electrons"] == 4 and got["nbands"] == 6


def test_unit_constants_codata_2018():
    u = O.units()
    # Bohr radius 0.529177210903 A, Hartree 27.211386245988 eV, k_B 3.166811563e-6 Ha/K; the
    # reference's mu_0 = 4 pi 1e-7 (not the 2019 SI value) moves them by ~1e-10
    assert 1.0 / u["A"] == pytest.approx(0.529177210903, rel=1e-8)
    assert 1.0 / u["eV"] == pytest.approx(27.211386245988, rel=1e-8)
    assert u["K"] == pytest.approx(3.166811563e-6, rel=1e-8)
    import derek_gb300 as dg  # noqa: F401


def test_system_from_info(tmp_path):
    import derek_gb300 as dg
    p = tmp_path / "sys.info"
    p.write_text(CASES["basic"])
    s = dg.SystemSpec.from_info(p)
    ref = O.read_info(p)
    assert np.allclose(s.cell, np.asarray(ref["cell"]).reshape(3, 3, order="F"), rtol=0, atol=0)
    assert s.ecut == ref["cut_off_energy"] and s.nbands == 12 and s.nelec == 8.0
    assert s.kT == ref["electronic_temp"] and len(s.kpts) == 8
    p.write_text("electronic_temp : 0\n" + LATTICE)
    with pytest.raises(ValueError):
        dg.SystemSpec.from_info(p)
