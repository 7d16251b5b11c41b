"""derek_gb300.driver: a .info seed run end to end as program derek runs it
(read the parameters, build the external potential, SCF, the dos task,
write the files state_finalise writes).

CPU: the external potentials against the oracle's point-by-point
restatement of pot_external_pot (Source/pot.f90:128-166), quirks included.
GPU: runs of small seeds: the SCF equals a direct handle run, the files read
back as the handle's state, the DOS integrates to the band count, and a
uniform field gives a spinor run whose moment opposes the field.
"""
import os

import numpy as np
import pytest

LATTICE = "$DATA LATTICE\n6.0 0.0 0.0\n0.0 6.0 0.0\n0.0 0.0 6.0\n$ENDDATA LATTICE\n"
BASE = ("unit_energy : Ha\nunit_length : bohr\ncut_off_energy : 4.0\nn_electrons : 2\nconduction_bands : 4\n"
        "electronic_temp : 6000\nmax_scf : 80\nenergy_tol : 1e-10\n")


def write_seed(tmp_path, name, extra):
    seed = str(tmp_path / name)
    with open(seed + ".info", "w") as f:
        f.write(BASE + extra + LATTICE)
    return seed


@pytest.mark.parametrize("extra", [
    "external_pot : jelly\n",
    "external_pot : finite_barrier\nfinite_barrier_height : 2.0\nfinite_barrier_width : 0.6 0.4 0.5\n",
    "external_pot : periodic_pot\nperiodic_pot_amp : 1.5\nperiodic_pot_grid : 1 2 3\n",
    "external_pot : jelly\nunit_bfield : agr\next_bfield : 0.1 -0.2 0.3\n",
])
def test_external_potential_matches_oracle(oracle, tmp_path, extra):
    import derek_gb300 as dg
    from derek_gb300 import driver
    seed = write_seed(tmp_path, "pot", extra)
    p = dg.read_info(seed + ".info")
    n_fine = (10, 8, 6)
    got = driver.external_potential(p, n_fine)
    ref = oracle.external_nc_pot(p, n_fine)
    assert np.max(np.abs(got - ref)) < 1e-15
    assert driver._spinor_needed(got) == bool(np.any(np.asarray(p["ext_bfield"])))


@pytest.mark.gpu
def test_run_finite_barrier_dos_and_files(tmp_path):
    import derek_gb300 as dg
    from derek_gb300 import driver
    seed = write_seed(tmp_path, "fb",
                      "external_pot : finite_barrier\nfinite_barrier_height : -3.0\n"
                      "finite_barrier_width : 0.5 0.5 0.5\ntask : dos\ndos_kpt_mp_grid : 2 2 2\n"
                      "output_level : all\nwrite_xsf : true\n")
    out = driver.run(seed, precision=dg.DEREK_PREC_FP64)
    rep = out["report"]
    assert rep["converged"] and out["nspinor"] == 1
    p = dg.read_info(seed + ".info")
    nc = driver.external_potential(p, out["n_fine"])
    spec = driver.system_from_params(p, nc, 1)
    with dg.Handle(spec) as h:
        r = h.electronic_scf(max_scf=80, etol=1e-10)[0]
        rho = h.density()
    assert abs(r["free_energy"] - rep["free_energy"]) < 1e-10
    names = set(out["files"])
    assert {"fb-FB.potex", "fb.pot", "fb.den", "fb.wvfn", "fb-V.xsf", "fb-FB-V.xsf"} <= names
    nr = int(np.prod(out["n_fine"]))
    charge, _ = dg.read_den(seed + ".den", out["n_std"], nr)
    assert np.max(np.abs(charge.real - rho)) < 1e-9
    assert np.array_equal(dg.read_pot(os.path.join(tmp_path, "fb-FB.potex"), out["n_std"], nr), nc)
    e, d = out["dos"]
    integral = float(np.sum((d[1:] + d[:-1]) * np.diff(e)) / 2.0)
    assert abs(integral - 2 * p["nbands"]) < 1e-3 * p["nbands"]


@pytest.mark.gpu
def test_run_uniform_field_is_spinor(tmp_path):
    import derek_gb300 as dg
    from derek_gb300 import driver
    seed = write_seed(tmp_path, "b", "external_pot : jelly\nunit_bfield : agr\next_bfield : 0.0 0.0 0.4\n"
                                     "write_density : true\n")
    out = driver.run(seed, precision=dg.DEREK_PREC_FP64)
    assert out["nspinor"] == 2 and out["report"]["converged"]
    nr = int(np.prod(out["n_fine"]))
    _, spin = dg.read_den(seed + ".den", out["n_std"], nr)
    moment = spin.real.sum(axis=0)
    assert moment[2] < 0 and abs(moment[0]) < 1e-8 * abs(moment[2]) and abs(moment[1]) < 1e-8 * abs(moment[2])
