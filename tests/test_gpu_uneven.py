"""Sixteen systems of the uneven 256-system batch (systems 64..79: grids
32^3 to 72^3, 2 to 18 k-points, 4 to 60 electrons) in one handle, against
the FP64 oracle's converged states of three of them
(tests/golden/make_uneven_golden.py).

FP64 path: free energy, energy, Fermi level and eigenvalues within 1e-8 Ha,
density within 1e-7 (relative L2 on the stored points); every system of the
slice converges.  Mixed path: |dF| / N_e < 1e-6 Ha per electron.  The
mixed SCF stops at |dF| < 3e-8 Ha per electron here, below the benchmark's
1e-7: the benchmark compares two runs stopped by the same rule, this test
compares with the oracle's fixed point, and at 1e-7 the stopping rule alone
leaves a system up to ~1e-6 Ha/e from it (measured: system 71 at 1.0e-6).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
SLICE = list(range(64, 80))


def _batch():
    from derek_gb300 import workloads
    systems, mix = workloads.params("uneven256")
    return [systems[i] for i in SLICE], mix


@pytest.mark.parametrize("precision", [0, 1])
def test_uneven_slice_matches_oracle(precision):
    import derek_gb300 as dg
    from derek_gb300 import workloads
    g = dict(np.load(os.path.join(GOLDEN, "uneven_slice.npz")))
    systems, mix = _batch()
    opts = dict(mix)
    if precision == 0:
        opts.update(density_tol=1e-9)
        etol, per_e = 1e-11, 0
    else:
        # CUDA-core subspace products, as the autotuner picks for subspaces
        # below 64 bands: with the split-BF16 tensor cores system 71 (36
        # electrons in a 9-bohr cell) lands 1.0e-6 Ha/e from the oracle,
        # with CUDA cores 2.6e-7 (measured)
        opts.update(density_tol=0.0, use_tensor_cores=0)
        etol, per_e = 3e-8, 1
    with dg.Handle(workloads.to_specs(systems), precision=precision, etol_per_electron=per_e, **opts) as h:
        rep = h.electronic_scf(max_scf=300, etol=etol)
        got = {i: (rep[SLICE.index(i)], h.eigenvalues(SLICE.index(i)), h.density(SLICE.index(i)))
               for i in g["systems"]}
    assert all(r["converged"] for r in rep), [r["iterations"] for r in rep]
    for i in g["systems"]:
        r, eig, rho = got[i]
        ne = systems[SLICE.index(i)]["nelec"]
        if precision == 0:
            assert abs(r["free_energy"] - g[f"free_energy_{i}"]) < 1e-8, (i, r["free_energy"], g[f"free_energy_{i}"])
            assert abs(r["energy"] - g[f"energy_{i}"]) < 1e-8
            assert abs(r["efermi"] - g[f"efermi_{i}"]) < 1e-8
            assert np.max(np.abs(eig - g[f"eig_{i}"])) < 1e-8
            ref = g[f"density_{i}"]
            sub = rho[::int(g["density_stride"])]
            assert np.linalg.norm(sub - ref) / np.linalg.norm(ref) < 1e-7
        else:
            assert abs(r["free_energy"] - g[f"free_energy_{i}"]) / ne < 1e-6, i
