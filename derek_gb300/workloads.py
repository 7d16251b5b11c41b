"""Seeded synthetic inputs with the shapes of the benchmark workloads.

Every workload is a cubic cell holding a uniform jellium background plus
attractive Gaussian wells (depth U[1,3] Ha, width U[0.8,1.5] bohr, centres
uniform in the cell), spin-unpolarised, Fermi-Dirac smearing kT = 0.01 Ha:

  gamma_8e     L=10 bohr, Ecut=10 Ha, grid 32^3, Gamma only, 8 electrons in
               8 bands, 4 wells, Pulay alpha=0.3
  kpts64       L=16, Ecut=20, grid 72^3, 4x4x4 Monkhorst-Pack (64 k-points),
               64 electrons in 80 bands, 16 wells, Kerker + Pulay
  kpts64_k4    kpts64 with its first 4 k-points only (profiler captures)
  adjoint9k    L=12, Ecut=15, grid 48^3, Gamma + 2x2x2 (9 k-points), 16
               electrons in 20 bands, 8 wells
  uneven256    256 systems, L ~ U[8,20], Ecut=15, {2,3}-smooth grids, 2..64
               electrons, 1..27 k-points, 2..12 wells

The generator is numpy's PCG64 with the stated seed, so the inputs are the
same on every machine.

``params(name)`` returns the systems as plain dicts (cell, ecut, kpts,
nbands, nelec, kT, wells) and imports nothing from the package, so a CPU-only
caller can load this file on its own without the GPU library; the workload
functions and ``WORKLOADS`` return ``SystemSpec`` objects.
"""
from __future__ import annotations

import numpy as np


def mp_grid(n):
    """Monkhorst-Pack points k = i d - (1 + d)/2 (DEReK's io_kpoint_grid rule,
    Source/io.f90:2016-2031), x outermost."""
    out = []
    d = [1.0 / x for x in n]
    for a in range(1, n[0] + 1):
        for b in range(1, n[1] + 1):
            for c in range(1, n[2] + 1):
                out.append([a * d[0] - (1 + d[0]) / 2, b * d[1] - (1 + d[1]) / 2,
                            c * d[2] - (1 + d[2]) / 2])
    return np.array(out)


def wells(rng, count):
    c = rng.random((count, 3))
    dep = rng.uniform(1.0, 3.0, count)
    wid = rng.uniform(0.8, 1.5, count)
    return np.concatenate([c, dep[:, None], wid[:, None]], axis=1)


def _sys(L, ecut, kpts, nbands, nelec, w):
    return dict(cell=np.eye(3) * float(L), ecut=float(ecut), kpts=np.asarray(kpts, dtype=np.float64),
                nbands=int(nbands), nelec=float(nelec), kT=0.01, wells=w)


def _gamma_8e(seed=1):
    rng = np.random.default_rng(seed)
    return [_sys(10.0, 10.0, [[0, 0, 0]], 8, 8.0, wells(rng, 4))], dict(mix_alpha=0.3, kerker_q0=0.0)


def _kpts64(seed=2):
    rng = np.random.default_rng(seed)
    # Kerker + Pulay at alpha = 0.6, q0 = 0.8 / bohr: the middle of the
    # plateau of 9 SCF iterations in a measured grid (alpha 0.3-0.8, q0
    # 0.5-1.6, 8 or 12 Pulay pairs; both paths, filter degree 6).  alpha =
    # 0.3 took 12 iterations on the mixed and on the FP64 path.
    return [_sys(16.0, 20.0, mp_grid((4, 4, 4)), 80, 64.0, wells(rng, 16))], \
        dict(mix_alpha=0.6, kerker_q0=0.8)


def _kpts64_k4(seed=2):
    """kpts64 cut to its first 4 k-points: the same kernels on a case small
    enough for a full profiler capture and for the oracle's fixture."""
    systems, mix = _kpts64(seed)
    systems[0]["kpts"] = systems[0]["kpts"][:4].copy()
    return systems, mix


def _adjoint9k(seed=3):
    rng = np.random.default_rng(seed)
    k = np.concatenate([[[0.0, 0.0, 0.0]], mp_grid((2, 2, 2))])
    return [_sys(12.0, 15.0, k, 20, 16.0, wells(rng, 8))], dict(mix_alpha=0.3, kerker_q0=0.0)


def _uneven(count=256, seed=5):
    rng = np.random.default_rng(seed)
    systems = []
    for _ in range(count):
        L = rng.uniform(8.0, 20.0)
        ne = int(rng.integers(2, 65))
        ne += ne % 2
        nb = ne // 2 + max(4, ne // 8)
        while True:
            kg = tuple(int(x) for x in rng.integers(1, 4, 3))
            if np.prod(kg) <= 27:
                break
        systems.append(_sys(L, 15.0, mp_grid(kg), nb, float(ne),
                            wells(rng, int(rng.integers(2, 13)))))
    # plain Pulay over the last 4 pairs: many of these cells are large and
    # nearly empty (a few electrons bound in wells), where Kerker damping of
    # the long wavelengths slows convergence; measured on the mixed path, 256
    # of 256 systems converge (mean 19.6 iterations) against 253 with Kerker
    # q0 = 0.8 and 8 pairs (mean 25.0)
    return systems, dict(mix_alpha=0.3, kerker_q0=0.0, pulay_history=4)


_PARAMS = {"gamma_8e": _gamma_8e, "kpts64": _kpts64, "kpts64_k4": _kpts64_k4, "adjoint9k": _adjoint9k,
           "uneven256": _uneven}


def params(name, **kw):
    """(systems as plain dicts, mixing options) of a named workload."""
    return _PARAMS[name](**kw)


def to_specs(systems):
    from . import SystemSpec, DEREK_GRID_SMOOTH23
    return [SystemSpec(s["cell"], s["ecut"], s["kpts"], s["nbands"], s["nelec"], kT=s["kT"],
                       wells=s["wells"], grid_policy=DEREK_GRID_SMOOTH23) for s in systems]


def _specs(name):
    def make(**kw):
        systems, mix = params(name, **kw)
        return to_specs(systems), mix
    make.__name__ = name
    make.__doc__ = _PARAMS[name].__doc__
    return make


gamma_8e = _specs("gamma_8e")
kpts64 = _specs("kpts64")
kpts64_k4 = _specs("kpts64_k4")
adjoint9k = _specs("adjoint9k")
uneven = _specs("uneven256")

WORKLOADS = {"gamma_8e": gamma_8e, "kpts64": kpts64, "kpts64_k4": kpts64_k4, "adjoint9k": adjoint9k,
             "uneven256": uneven}
