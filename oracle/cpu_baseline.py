"""CPU timing of the oracle on a bounded sample of an SCF workload.

TEST INFRASTRUCTURE ONLY: used by bench.py's CPU-baseline leg and its
reference arm (the DEReK reference has no working SCF and cannot be built on
the benchmark host, so the FP64 numpy restatement stands in for it).

The sample is one Chebyshev-filtered subspace iteration of one k-point with
the same structure the GPU solver runs per SCF iteration: `degree` filtered
H.psi block applications, one more H.psi for Rayleigh-Ritz, the overlap
Cholesky orthonormalisation and the dense subspace eigensolve.  The
ground-state rate is this per-(k-point, iteration) cost scaled by the number
of k-points and by the H.psi work of a full SCF, both stated by the caller.
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import derek_oracle as O


def _system_from(spec):
    cell = np.asarray(spec["cell"], dtype=np.float64)
    n_std, n_fine = O.grid_sizes(cell, spec["ecut"], 2.0, "smooth23")
    kpts = np.asarray(spec["kpts"], dtype=np.float64).reshape(-1, 3)
    wk = np.full(len(kpts), 1.0 / len(kpts))
    wells = np.asarray(spec["wells"], dtype=np.float64).reshape(-1, 5)
    vext = O.vext_jellium_wells(cell, n_fine, spec["nelec"], wells)
    return O.System(cell, spec["ecut"], n_fine, n_std, kpts, wk, spec["nbands"], spec["nelec"],
                    spec["kT"], vext, wells)


def subspace_iteration(sys: O.System, ik: int, degree: int, seed: int = 0) -> float:
    """Seconds for one filtered subspace iteration of k-point ik (FP64 numpy)."""
    import scipy.linalg as sla
    kb = O.KBasis(sys, ik)
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((sys.nbands, kb.npw)) + 0j
    v = sys.vext
    t0 = time.perf_counter()
    # filter with fixed bounds (the arithmetic, not the convergence, is timed)
    a0, a, b = -1.0, 0.5, sys.ecut + float(v.max())
    e, c = 0.5 * (b - a), 0.5 * (b + a)
    s1 = e / (a0 - c)
    Y = (O.apply_h(sys, kb, v, X) - c * X) * (s1 / e)
    s = s1
    for _ in range(1, degree):
        sn = 1.0 / (2.0 / s1 - s)
        Yn = 2.0 * sn / e * (O.apply_h(sys, kb, v, Y) - c * Y) - s * sn * X
        X, Y, s = Y, Yn, sn
    S = Y.conj() @ Y.T
    L = np.linalg.cholesky(S)
    Xo = sla.solve_triangular(L, Y, lower=True)
    HX = O.apply_h(sys, kb, v, Xo)
    Hs = Xo.conj() @ HX.T
    w, U = np.linalg.eigh(0.5 * (Hs + Hs.conj().T))
    _ = U.T @ Xo
    return time.perf_counter() - t0


def _worker(args):
    spec, ik, degree = args
    sys = _system_from(spec)
    return subspace_iteration(sys, ik, degree)


def sample(spec: dict, degree: int, kpoints: int = 1, workers: int = 1) -> dict:
    """Time `kpoints` k-point iterations, spread over `workers` processes
    (started with spawn).  Returns seconds per (k-point, iteration) averaged
    over the sample, wall seconds, and the worker count actually used."""
    jobs = [(spec, ik % len(spec["kpts"]), degree) for ik in range(kpoints)]
    t0 = time.perf_counter()
    if workers <= 1:
        times = [_worker(j) for j in jobs]
    else:
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        with ctx.Pool(workers) as pool:
            times = pool.map(_worker, jobs)
    wall = time.perf_counter() - t0
    return {"per_k_iteration_s": float(np.mean(times)), "wall_s": wall,
            "workers": workers, "kpoints": kpoints,
            "throughput_k_iterations_per_s": kpoints / wall}


def cores() -> int:
    return os.cpu_count() or 1
