"""Oracle fixtures for three systems of the uneven 256-system batch
(derek_gb300/workloads.py "uneven256", seed 5), for the GPU test that runs
systems 64..79 of the batch in one handle (every grid class 32^3 ... 72^3):

  system 65  L=9.68 bohr, 36^3, 2 k-points, 32 electrons in 20 bands
  system 71  L=9.07 bohr, 32^3, 3 k-points, 36 electrons in 22 bands
  system 73  L=13.55 bohr, 48^3, 8 k-points, 14 electrons in 11 bands

Each is solved with the FP64 oracle (Chebyshev-filtered eigensolver, Pulay
alpha 0.3 over 4 pairs, no Kerker: the batch's mixing) to |dF| < 1e-11 Ha and
max|n_out - n_in| < 1e-9.  uneven_slice.npz holds, per system, the
eigenvalues, occupations, Fermi level, energies and every 7th point of the
density.
Usage: python tests/golden/make_uneven_golden.py
"""
import importlib.util
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import derek_oracle as O  # noqa: E402

SYSTEMS = [65, 71, 73]
STRIDE = 7


def main():
    spec = importlib.util.spec_from_file_location("wl", os.path.join(ROOT, "derek_gb300", "workloads.py"))
    wl = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(wl)
    batch, mix = wl.params("uneven256")
    out = {"systems": np.array(SYSTEMS), "density_stride": STRIDE}
    for i in SYSTEMS:
        p = batch[i]
        s = O.make_system(p["cell"][0, 0], p["ecut"], p["nelec"], p["nbands"], p["wells"], kpts=p["kpts"],
                          kT=p["kT"])
        t = time.time()
        r = O.scf(s, max_scf=300, etol=1e-11, rtol=1e-9, alpha=mix["mix_alpha"], history=mix["pulay_history"],
                  q0=mix["kerker_q0"], solver="filtered", workers=int(os.environ.get("ORACLE_THREADS", "2")))
        print(i, "converged" if r.converged else "NOT converged", r.iterations, f"{time.time() - t:.0f}s",
              f"F={r.free_energy:.12f}", flush=True)
        assert r.converged
        for key, val in (("eig", r.eigenvalues), ("occ", r.occupations), ("efermi", r.efermi),
                         ("energy", r.energy), ("free_energy", r.free_energy),
                         ("density", r.density[::STRIDE]), ("n_fine", np.array(s.n_fine))):
            out[f"{key}_{i}"] = val
    np.savez_compressed(os.path.join(HERE, "uneven_slice.npz"), **out)


if __name__ == "__main__":
    main()
