"""Failure paths on the GPU, made without faulting it:

* a tensor-core pipeline wait that runs out (its try limit lowered with
  derek_gpu_set_wait_limit): the overlap and the SCF report
  DEREK_ERR_TIMEOUT, and the same handle then works once the limit is back;
* linearly dependent start vectors (two equal bands restored with
  init_vectors = 2): the Cholesky orthonormalisation reports
  DEREK_ERR_CHOLESKY, and the same handle then converges from valid ones;
* a restart from stored wavefunctions (init_vectors = 2, the reference's
  state_write keeps model%wfn) reaches the oracle's ground state in fewer
  iterations than a cold start.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _fixture():
    return dict(np.load(os.path.join(GOLDEN, "scf_kpts.npz")))


def _handle(oracle, d, precision, **opts):
    import derek_gb300 as dg
    cell = d["cell"]
    nf = tuple(int(x) for x in d["n_fine"])
    vext = oracle.vext_jellium_wells(cell, nf, float(d["nelec"]), d["wells"])
    spec = dg.SystemSpec(cell, float(d["ecut"]), d["kpts"], int(d["nbands"]), float(d["nelec"]),
                         kT=float(d["kT"]), wk=d["wk"], vext=vext, n_fine=nf, inv_cell=oracle.inv_cell(cell))
    kw = dict(mix_alpha=0.3, kerker_q0=float(d["q0"]), pulay_history=8, density_tol=1e-10)
    kw.update(opts)
    return dg.Handle(spec, precision=precision, **kw)


def test_tensor_core_wait_timeout_is_reported_and_the_handle_recovers(oracle):
    import derek_gb300 as dg
    d = _fixture()
    rng = np.random.default_rng(3)
    with _handle(oracle, d, dg.DEREK_PREC_MIXED, use_tensor_cores=2, density_tol=0.0) as h:
        npw = h.npw(0, 0)
        psi = rng.standard_normal((int(d["nbands"]), npw)) + 1j * rng.standard_normal((int(d["nbands"]), npw))
        h.set_wfn(psi, 0, 0)
        try:
            assert dg.lib.derek_gpu_set_wait_limit(0) == 0
            with pytest.raises(dg.DerekError) as e:
                h.wave_dot(0, 0)
            assert e.value.status == dg._abi.DEREK_ERR_TIMEOUT
            with pytest.raises(dg.DerekError) as e:
                h.electronic_scf(max_scf=50, etol=1e-7)
            assert e.value.status == dg._abi.DEREK_ERR_TIMEOUT
        finally:
            assert dg.lib.derek_gpu_set_wait_limit(-1) == 0
        h.set_wfn(psi, 0, 0)
        s = h.wave_dot(0, 0)
        p32 = psi.astype(np.complex64).astype(np.complex128)
        ref = p32.conj() @ p32.T
        assert np.max(np.abs(s - ref)) / np.max(np.abs(ref)) < 5e-5
        # the mixed path stops at 1e-7 Ha, as the other mixed-precision tests
        rep = h.electronic_scf(max_scf=300, etol=1e-7)[0]
    assert rep["converged"]
    assert abs(rep["free_energy"] - float(d["free_energy"])) / float(d["nelec"]) < 1e-6


def test_duplicated_start_bands_report_cholesky_and_the_handle_recovers(oracle):
    import derek_gb300 as dg
    d = _fixture()
    nb = int(d["nbands"])
    with _handle(oracle, d, dg.DEREK_PREC_FP64, init_vectors=2, buffer_bands=2) as h:
        rng = np.random.default_rng(5)
        good = []
        for k in range(len(d["kpts"])):
            npw = h.npw(0, k)
            psi = rng.standard_normal((nb, npw)) + 1j * rng.standard_normal((nb, npw))
            good.append(psi.copy())
            if k == 1:
                psi[3] = psi[2]          # two equal bands: S is singular
            h.set_wfn(psi, 0, k)
        with pytest.raises(dg.DerekError) as e:
            h.electronic_scf(max_scf=20, etol=1e-9)
        assert e.value.status == dg._abi.DEREK_ERR_CHOLESKY
        for k, psi in enumerate(good):
            h.set_wfn(psi, 0, k)
        rep = h.electronic_scf(max_scf=300, etol=1e-12)[0]
    assert rep["converged"]
    assert abs(rep["free_energy"] - float(d["free_energy"])) < 1e-8


def test_restart_from_stored_wavefunctions(oracle):
    d = _fixture()
    with _handle(oracle, d, 0, init_vectors=1) as h:
        cold = h.electronic_scf(max_scf=300, etol=1e-12)[0]
        wfn = [h.get_wfn(0, k) for k in range(len(d["kpts"]))]
        rho = h.density()
    with _handle(oracle, d, 0, init_vectors=2) as h2:
        for k, psi in enumerate(wfn):
            h2.set_wfn(psi, 0, k)
        h2.set_start_density(rho)
        warm = h2.electronic_scf(max_scf=300, etol=1e-12)[0]
    assert cold["converged"] and warm["converged"]
    assert warm["iterations"] < cold["iterations"]
    assert abs(warm["free_energy"] - float(d["free_energy"])) < 1e-8


def test_primitives_after_a_converged_scf(oracle):
    """A converged SCF masks its systems off on the device; the overlap and
    H.psi entry points still work on them afterwards (numpy conj(X) X^T at
    1e-12, the oracle's H.psi in the SCF's last potential at 1e-11)."""
    d = _fixture()
    nb = int(d["nbands"])
    with _handle(oracle, d, 0) as h:
        rep = h.electronic_scf(max_scf=300, etol=1e-12)[0]
        assert rep["converged"]
        vloc = h.get_vloc()
        rng = np.random.default_rng(8)
        k = 1
        npw = h.npw(0, k)
        psi = rng.standard_normal((nb, npw)) + 1j * rng.standard_normal((nb, npw))
        h.set_wfn(psi, 0, k)
        s = h.wave_dot(0, k)
        hpsi = h.pot_apply_wfn(0, k)
    ref = psi.conj() @ psi.T
    assert np.max(np.abs(s - ref)) / np.max(np.abs(ref)) < 1e-12
    cell = d["cell"]
    nf = tuple(int(x) for x in d["n_fine"])
    sysm = oracle.System(cell, float(d["ecut"]), nf, oracle.grid_sizes(cell, float(d["ecut"]))[0], d["kpts"],
                         d["wk"], nb, float(d["nelec"]), float(d["kT"]), vloc, d["wells"])
    href = oracle.apply_h(sysm, oracle.KBasis(sysm, k), vloc, psi)
    assert np.max(np.abs(hpsi - href)) / np.max(np.abs(href)) < 1e-11
