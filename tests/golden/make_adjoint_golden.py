"""Central finite differences of the FP64 CPU oracle on the adjoint-gradient
workload (BASELINE config 4), stored as a fixture for the GPU adjoint test:

  adjoint9k.npz   cubic L=12 bohr, Ecut=15 Ha, 48^3 grid, Gamma + 2x2x2
                  Monkhorst-Pack (9 k-points), 16 electrons in 20 bands,
                  kT=0.01 Ha, jellium + 8 Gaussian wells from seed 3 (depth,
                  width and centre of each are parameters), Pulay alpha=0.3.
                  The target density comes from a second well set (seed 33).

For three parameters p (depth of well 0, width of well 3, x-centre of well 5)
the oracle runs the SCF at p + h and p - h (h = 1e-5, warm-started from the
converged base state) and stores
  fd_loss = (L(p+h) - L(p-h)) / 2h,  L = sum (n - n_target)^2 dV,
  fd_free = (F(p+h) - F(p-h)) / 2h   (the Hellmann-Feynman derivative),
with every SCF converged to |dF| < 1e-13 Ha and max|n_out - n_in| < 1e-11
(Chebyshev-filtered eigensolver, two passes per iteration, the last
iteration's eigenproblem solved to residuals of 1e-12).  Also stored: the base
and target free energies, L at the base point, and every 11th point of the
base and target densities.
Usage: python tests/golden/make_adjoint_golden.py
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import derek_oracle as O  # noqa: E402

L_CELL, ECUT, NB, NE = 12.0, 15.0, 20, 16.0
H = 1e-5
PARAMS = [(0, 3), (3, 4), (5, 0)]   # (well, column): columns cx, cy, cz, depth, width
STRIDE = 11
KW = dict(max_scf=300, etol=1e-13, rtol=1e-11, alpha=0.3, history=8, q0=0.0, solver="filtered",
          eig_tol=1e-12, workers=os.cpu_count(), passes=2)


def system(wells):
    kpts = np.concatenate([[[0.0, 0.0, 0.0]], O.mp_kpoints((2, 2, 2))])
    return O.make_system(L_CELL, ECUT, NE, NB, wells, kpts=kpts, kT=0.01)


def run(wells, **kw):
    t = time.time()
    keep = {}
    s = system(wells)
    r = O.scf(s, keep=keep, **KW, **kw)
    print(f"  F={r.free_energy:.14f} it={r.iterations} conv={r.converged} {time.time() - t:.0f}s", flush=True)
    assert r.converged
    return s, r, keep


def main():
    wells = O.random_wells(np.random.default_rng(3), 8)
    target_wells = O.random_wells(np.random.default_rng(33), 8)
    print("target", flush=True)
    st, rt, _ = run(target_wells)
    n_t = rt.density
    print("base", flush=True)
    s0, r0, keep0 = run(wells)
    dv = s0.volume / s0.nr
    loss = lambda r: float(np.sum((r.density - n_t) ** 2) * dv)
    fd_loss, fd_free = [], []
    for (w, c) in PARAMS:
        vals = []
        for sgn in (1, -1):
            wp = wells.copy()
            wp[w, c] += sgn * H
            print(f"well {w} col {c} {'+' if sgn > 0 else '-'}h", flush=True)
            _, r, _ = run(wp, nin0=r0.density, blocks0=keep0["blocks"])
            vals.append((loss(r), r.free_energy))
        fd_loss.append((vals[0][0] - vals[1][0]) / (2 * H))
        fd_free.append((vals[0][1] - vals[1][1]) / (2 * H))
        print(f"  dL/dp={fd_loss[-1]:.10e} dF/dp={fd_free[-1]:.10e}", flush=True)
    np.savez_compressed(os.path.join(HERE, "adjoint9k.npz"), cell=s0.cell, ecut=ECUT, n_fine=np.array(s0.n_fine),
                        kpts=s0.kpts, wk=s0.wk, nbands=NB, nelec=NE, kT=0.01, wells=wells,
                        target_wells=target_wells, h=H, params=np.array(PARAMS), fd_loss=np.array(fd_loss),
                        fd_free=np.array(fd_free), loss=loss(r0), free_energy=r0.free_energy,
                        target_free_energy=rt.free_energy, density_stride=STRIDE,
                        density=r0.density[::STRIDE], target_density=n_t[::STRIDE])


if __name__ == "__main__":
    main()
