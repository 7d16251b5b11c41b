"""The autotuner (derek_gpu_autotune): its cache format and candidate lists
on the CPU, and on the GPU that a tuned handle reaches the same ground state
(every candidate plan computes the same result) and that a second handle
takes its plan from the cache."""
import ctypes
import json
import os

import numpy as np
import pytest


def _lib():
    import derek_gb300 as dg
    return dg.lib


def _radix_candidates(n):
    buf = ctypes.create_string_buffer(4096)
    assert _lib().derek_host_radix_candidates(n, buf, len(buf)) == 0
    v = buf.value.decode()
    return [] if not v else v.split(";")


@pytest.mark.parametrize("n", [24, 27, 30, 32, 36, 42, 48, 54, 64, 65, 72, 96, 128])
def test_radix_candidates_factor_the_length(n):
    cands = _radix_candidates(n)
    assert cands, n
    assert len(set(cands)) == len(cands)
    for c in cands:
        r = [int(x) for x in c.split("x")]
        assert np.prod(r) == n
        assert set(r) <= {2, 3, 4, 5, 7, 8, 11, 13}
        assert len(r) <= 8


def test_radix_candidates_reject_large_primes():
    assert _radix_candidates(34) == []   # 17 has no radix


def test_cache_round_trip():
    cache = {"NVIDIA GB300 (152 SMs)": {"fft n=72": "8x3x3", "lines prec=mixed n=72": "fixed",
                                          "rows prec=mixed n=72 m=16": "tight",
                                          "overlap prec=mixed nb=84 npw=17529 nks=64": "tc 4096",
                                          "jacobi nb=84 nks=64": "pair"},
             "other \"gpu\" (8 SMs)": {}}
    text = json.dumps(cache)
    buf = ctypes.create_string_buffer(1 << 16)
    assert _lib().derek_host_tune_cache_normalise(text.encode(), buf, len(buf)) == 0
    assert json.loads(buf.value.decode()) == cache
    # the library's own layout reads back to the same object
    again = ctypes.create_string_buffer(1 << 16)
    assert _lib().derek_host_tune_cache_normalise(buf.value, again, len(again)) == 0
    assert again.value == buf.value
    assert _lib().derek_host_tune_cache_normalise(b'{"a": {"k": 3}}', buf, len(buf)) != 0
    assert _lib().derek_host_tune_cache_normalise(b'{"a": {"k": "v"}', buf, len(buf)) != 0


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_tuned_handle_reaches_the_oracle_ground_state(oracle, tmp_path, precision):
    """FP64: the tuned plan keeps F, E and the eigenvalues within 1e-8 Ha of
    the oracle fixture; mixed: |dF| / N_e < 1e-6.  A second handle reads the
    same plan from the cache file."""
    import derek_gb300 as dg
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "scf_kpts.npz")))
    cell = d["cell"]
    nf = tuple(int(x) for x in d["n_fine"])
    vext = oracle.vext_jellium_wells(cell, nf, float(d["nelec"]), d["wells"])
    spec = dg.SystemSpec(cell, float(d["ecut"]), d["kpts"], int(d["nbands"]), float(d["nelec"]),
                         kT=float(d["kT"]), wk=d["wk"], vext=vext, n_fine=nf, inv_cell=oracle.inv_cell(cell))
    # the mixed path stops at 1e-7 Ha (its FP32 H.psi cannot resolve 1e-12)
    kw = dict(mix_alpha=0.3, kerker_q0=float(d["q0"]), pulay_history=8,
              density_tol=1e-10 if precision == 0 else 0.0)
    cache = tmp_path / "tune.json"
    with dg.Handle(spec, precision=precision, **kw) as h:
        plan = h.autotune(cache)
        assert plan["source"] == "tuned"
        rep = h.electronic_scf(max_scf=300, etol=1e-12 if precision == 0 else 1e-7)[0]
        eig = h.eigenvalues()
    assert rep["converged"]
    if precision == 0:
        assert abs(rep["free_energy"] - d["free_energy"]) < 1e-8
        assert abs(rep["energy"] - d["energy"]) < 1e-8
        assert np.max(np.abs(eig - d["eig"])) < 1e-8
    else:
        assert abs(rep["free_energy"] - d["free_energy"]) / float(d["nelec"]) < 1e-6
    stored = json.loads(cache.read_text())
    assert len(stored) == 1 and any(k.startswith("fft n=") for k in next(iter(stored.values())))
    with dg.Handle(spec, precision=precision, **kw) as h2:
        plan2 = h2.autotune(cache)
    assert plan2["source"] == "cache"
    assert {k: v for k, v in plan2.items() if k != "source"} == {k: v for k, v in plan.items() if k != "source"}
