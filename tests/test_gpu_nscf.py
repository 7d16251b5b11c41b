"""Non-self-consistent eigenvalues (the bandstructure and dos tasks) against
the oracle's dense diagonalisation of H(k) in the same plane-wave basis and
potential (FP64 1e-8 Ha; mixed path 2e-5 Ha), and against the SCF's own
eigenvalues in its converged potential."""
import numpy as np
import pytest

from test_gpu_primitives import make_pair
from test_gpu_scf import load, make_handle

pytestmark = pytest.mark.gpu


def dense_eigenvalues(oracle, s, ik, v, nb):
    kb = oracle.KBasis(s, ik)
    h = oracle.apply_h(s, kb, v, np.eye(kb.npw, dtype=np.complex128))
    h = 0.5 * (h + h.conj().T)
    return np.linalg.eigvalsh(h)[:nb]


@pytest.mark.parametrize("precision,tol", [(0, 1e-8), (1, 2e-5)])
def test_nscf_matches_dense_oracle(oracle, precision, tol):
    import derek_gb300 as dg
    kpts = ((0.0, 0.0, 0.0), (0.1, 0.2, -0.3), (0.5, 0.0, 0.25))   # a short path
    s, spec = make_pair(oracle, kpts=kpts, nb=6, seed=7)
    rng = np.random.default_rng(8)
    v = s.vext + 0.2 * rng.standard_normal(s.nr)
    with dg.Handle(spec, precision=precision, cheb_degree=8, init_vectors=1) as h:
        h.set_vloc(v)
        # the mixed path stops at its FP32 noise floor
        (eig,), it = h.nscf(max_iter=300, eig_tol=1e-11 if precision == 0 else 2e-6)
    for ik in range(len(kpts)):
        ref = dense_eigenvalues(oracle, s, ik, v, 6)
        assert np.max(np.abs(eig[ik] - ref)) < tol, (ik, np.max(np.abs(eig[ik] - ref)))
    assert it > 0


def test_nscf_in_scf_potential_reproduces_scf_eigenvalues(oracle):
    """The converged SCF potential, handed to a second handle with the same
    k-points, gives back the SCF's eigenvalues; the DOS integrates to two
    electrons per band."""
    import derek_gb300 as dg
    d = load("scf_c1")
    with make_handle(oracle, d) as h:
        rep = h.electronic_scf(max_scf=300, etol=1e-12)[0]
        v = h.get_vloc()
        eig_scf = h.eigenvalues()
    assert rep["converged"]
    with make_handle(oracle, d, init_vectors=1, cheb_degree=8) as h2:
        h2.set_vloc(v)
        (eig,), _ = h2.nscf(max_iter=300, eig_tol=1e-11)
        e = np.linspace(eig.min() - 1.0, eig.max() + 1.0, 4001)
        dos = h2.dos(e, sigma=0.02)
    assert np.max(np.abs(eig - eig_scf)) < 1e-8, np.max(np.abs(eig - eig_scf))
    assert abs(np.trapezoid(dos, e) - 2 * int(d["nbands"])) < 1e-6
