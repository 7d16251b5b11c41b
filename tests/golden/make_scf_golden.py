"""Runs the FP64 CPU oracle SCF on seeded workloads and stores the converged
results as fixtures for the GPU parity tests:

  scf_c1.npz         cubic L=10 bohr, Ecut=10 Ha, 32^3 grid, Gamma only, 8
                     electrons in 8 bands, kT=0.01 Ha, jellium + 4 Gaussian
                     wells (depth U[1,3] Ha, width U[0.8,1.5] bohr), Pulay
                     alpha=0.3 (dense diagonalisation)
  scf_kpts.npz       cubic L=7, Ecut=6, 2x2x2 Monkhorst-Pack, 6 electrons in 8
                     bands, 3 wells, Kerker (q0=0.8) + Pulay (dense)
  scf_kpts64_k4.npz  the 64-k-point benchmark system (cubic L=16, Ecut=20 Ha,
                     72^3 grid, 64 electrons in 80 bands, 16 wells from seed 2,
                     Kerker + Pulay) on the first 4 of its 4x4x4 Monkhorst-Pack
                     k-points, solved with the oracle's Chebyshev-filtered
                     eigensolver (17,529 plane waves per k-point: too many for
                     a dense matrix), two filter passes per SCF iteration and
                     the last iteration's eigenproblem solved to 1e-9

Each file holds the inputs (cell, ecut, grid, k-points, wells) and the
converged eigenvalues, occupations, Fermi level, energies and output density
(|dF| < 1e-12 Ha and max|n_out - n_in| < 1e-11 for the small cases; 1e-11 Ha
and 1e-9 for the large one, whose density is stored on every 17th grid point
to keep the file small).
Usage: python tests/golden/make_scf_golden.py [case ...]   (default: all)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import derek_oracle as O  # noqa: E402

CASES = {
    "scf_c1": dict(L=10.0, ecut=10.0, nelec=8, nb=8, nwells=4, seed=1, kgrid=(1, 1, 1), q0=0.0),
    "scf_kpts": dict(L=7.0, ecut=6.0, nelec=6, nb=8, nwells=3, seed=2, kgrid=(2, 2, 2), q0=0.8),
    "scf_kpts64_k4": dict(L=16.0, ecut=20.0, nelec=64, nb=80, nwells=16, seed=2, kgrid=(4, 4, 4),
                          nk=4, q0=0.8, solver="filtered", etol=1e-11, rtol=1e-9, stride=17, buffer=24,
                          passes=2),
}


def run(name, c):
    rng = np.random.default_rng(c["seed"])
    wells = O.random_wells(rng, c["nwells"])
    kpts = O.mp_kpoints(c["kgrid"])[:c.get("nk")]
    s = O.make_system(c["L"], c["ecut"], c["nelec"], c["nb"], wells, kpts=kpts, kT=0.01)
    t = time.time()
    r = O.scf(s, max_scf=200, etol=c.get("etol", 1e-12), alpha=0.3, history=8, q0=c["q0"],
              rtol=c.get("rtol", 1e-11), solver=c.get("solver", "dense"), verbose="-v" in sys.argv,
              workers=os.cpu_count(), buffer=c.get("buffer", 8), passes=c.get("passes"))
    print(name, "converged" if r.converged else "NOT converged", r.iterations, "iterations",
          f"{time.time() - t:.1f}s", f"F={r.free_energy:.12f}", f"|R|={r.history[-1][4]:.1e}")
    stride = c.get("stride", 1)
    extra = {} if stride == 1 else dict(density_stride=stride,
                                        density_norm=np.linalg.norm(r.density),
                                        density_sum=r.density.sum())
    np.savez_compressed(os.path.join(HERE, name + ".npz"), cell=s.cell, ecut=s.ecut,
                        n_fine=np.array(s.n_fine), kpts=s.kpts, wk=s.wk, nbands=s.nbands,
                        nelec=s.nelec, kT=s.kT, wells=wells, q0=c["q0"],
                        eig=r.eigenvalues, occ=r.occupations, efermi=r.efermi, energy=r.energy,
                        free_energy=r.free_energy, density=r.density[::stride],
                        iterations=r.iterations, **extra)


if __name__ == "__main__":
    names = [a for a in sys.argv[1:] if not a.startswith("-")] or list(CASES)
    for n in names:
        run(n, CASES[n])
