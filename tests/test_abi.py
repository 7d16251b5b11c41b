"""The C-ABI library loads, exports every function include/derek_gpu.h
declares, and its host-side grid/sphere rules agree bit-for-bit with the
oracle's restatement of Source/basis.f90:87-149,257-309 (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "derek_gpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(derek_(?:gpu|host)_\w+)\s*\(", txt)))


def test_library_exports_header():
    import derek_gb300
    lib = ctypes.CDLL(derek_gb300.lib_path)
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_no_cpu_fallback_when_library_missing(tmp_path, monkeypatch):
    import importlib
    import derek_gb300._abi as abi
    monkeypatch.setattr(abi, "lib_path", str(tmp_path / "nope.so"))
    with pytest.raises(ImportError):
        abi._load()


@pytest.mark.parametrize("L,ecut", [(10.0, 10.0), (16.0, 20.0), (12.0, 15.0), (8.0, 15.0), (20.0, 15.0)])
def test_host_grid_sizes_match_oracle(oracle, L, ecut):
    import derek_gb300 as dg
    cell = np.eye(3) * L
    for pol, name in ((dg.DEREK_GRID_REFERENCE, "reference"), (dg.DEREK_GRID_SMOOTH23, "smooth23")):
        assert dg.host_grid_sizes(cell, ecut, 2.0, pol) == oracle.grid_sizes(cell, ecut, 2.0, name)


def test_host_prime_fact_matches_oracle(oracle):
    import derek_gb300 as dg
    for n in range(1, 400):
        assert dg.host_prime_fact(n) == oracle.prime_fact_round(n)


@pytest.mark.parametrize("cell,ecut,kgrid", [
    (np.eye(3) * 10.0, 10.0, (1, 1, 1)),
    (np.eye(3) * 16.0, 20.0, (4, 4, 4)),
    (np.eye(3) * 12.0, 15.0, (2, 2, 2)),
    (np.array([[7.0, 0.5, 0.0], [0.0, 6.5, 0.3], [0.2, 0.0, 8.0]]), 9.0, (2, 1, 3)),
])
def test_host_sphere_bit_exact(oracle, cell, ecut, kgrid):
    import derek_gb300 as dg
    ns, _ = oracle.grid_sizes(cell, ecut)
    inv = oracle.inv_cell(cell)
    for k in oracle.mp_kpoints(kgrid)[:8]:
        rows = dg.host_gsphere(inv, ecut, k, ns)
        ref, _, _ = oracle.gsphere(cell, ecut, k, ns, inv_cell_given=inv)
        assert np.array_equal(rows, ref)
