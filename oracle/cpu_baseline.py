"""CPU timing of the oracle on a bounded sample of an SCF workload.

TEST INFRASTRUCTURE ONLY: used by bench.py's CPU-baseline leg and its
reference arm (the DEReK reference has no working SCF and cannot be built on
the benchmark host, so the FP64 numpy restatement stands in for it).

The sample unit is one Chebyshev-filtered subspace iteration of one k-point
with the structure the GPU solver runs per SCF iteration: `degree` filtered
H.psi block applications, one more H.psi for Rayleigh-Ritz, the overlap
Cholesky orthonormalisation and the dense subspace eigensolve.  A pool of
worker processes (started with spawn, one per host core, each single
threaded) runs one such unit per worker per step; the caller scales the
measured step time to a ground state by the H.psi work of a full SCF.
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import derek_oracle as O

_CACHE = {}


def _system_from(spec):
    cell = np.asarray(spec["cell"], dtype=np.float64)
    n_std, n_fine = O.grid_sizes(cell, spec["ecut"], 2.0, "smooth23")
    kpts = np.asarray(spec["kpts"], dtype=np.float64).reshape(-1, 3)
    wk = np.full(len(kpts), 1.0 / len(kpts))
    wells = np.asarray(spec["wells"], dtype=np.float64).reshape(-1, 5)
    vext = O.vext_jellium_wells(cell, n_fine, spec["nelec"], wells)
    return O.System(cell, spec["ecut"], n_fine, n_std, kpts, wk, spec["nbands"], spec["nelec"],
                    spec["kT"], vext, wells)


def subspace_iteration(sys: O.System, kb: O.KBasis, X: np.ndarray, degree: int) -> float:
    """Seconds for one filtered subspace iteration of one k-point (FP64)."""
    import scipy.linalg as sla
    v = sys.vext
    t0 = time.perf_counter()
    # filter with fixed bounds (the arithmetic, not the convergence, is timed)
    a0, a, b = -1.0, 0.5, sys.ecut + float(v.max())
    e, c = 0.5 * (b - a), 0.5 * (b + a)
    s1 = e / (a0 - c)
    Y = (O.apply_h_block(sys, kb, v, X, workers=1) - c * X) * (s1 / e)
    s = s1
    for _ in range(1, degree):
        sn = 1.0 / (2.0 / s1 - s)
        Yn = 2.0 * sn / e * (O.apply_h_block(sys, kb, v, Y, workers=1) - c * Y) - s * sn * X
        X, Y, s = Y, Yn, sn
    S = Y.conj() @ Y.T
    L = np.linalg.cholesky(S)
    Xo = sla.solve_triangular(L.conj(), Y, lower=True)
    HX = O.apply_h_block(sys, kb, v, Xo, workers=1)
    Hs = Xo.conj() @ HX.T
    w, U = np.linalg.eigh(0.5 * (Hs + Hs.conj().T))
    _ = U.T @ Xo
    return time.perf_counter() - t0


def _worker(args):
    spec_key, spec, ik, degree = args
    key = (spec_key, ik)
    if key not in _CACHE:
        if spec_key not in _CACHE:
            _CACHE[spec_key] = _system_from(spec)
        sys = _CACHE[spec_key]
        kb = O.KBasis(sys, ik)
        X = np.random.default_rng(ik).standard_normal((sys.nbands, kb.npw)) + 0j
        _CACHE[key] = (kb, X)
    sys = _CACHE[spec_key]
    kb, X = _CACHE[key]
    return subspace_iteration(sys, kb, X, degree)


def _single_thread_env():
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[v] = "1"


class Sampler:
    """A spawn pool of `workers` single-threaded processes; `step()` runs one
    subspace iteration of a different k-point in every worker and returns
    the wall seconds of the step (the slowest worker's unit plus the
    dispatch).  The first step of each worker also builds its system and
    sphere, so callers warm up before timing."""

    def __init__(self, spec: dict, degree: int, workers: int):
        import multiprocessing as mp
        self.spec, self.degree, self.workers = spec, degree, max(1, int(workers))
        self.nk = len(np.asarray(spec["kpts"]).reshape(-1, 3))
        saved = {v: os.environ.get(v) for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
        _single_thread_env()
        self.pool = mp.get_context("spawn").Pool(self.workers)
        for v, x in saved.items():
            if x is None:
                os.environ.pop(v, None)
            else:
                os.environ[v] = x

    def step(self) -> float:
        jobs = [(id(self), self.spec, i % self.nk, self.degree) for i in range(self.workers)]
        t0 = time.perf_counter()
        self.pool.map(_worker, jobs, chunksize=1)
        return time.perf_counter() - t0

    def close(self):
        self.pool.close()
        self.pool.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def cores() -> int:
    return os.cpu_count() or 1
