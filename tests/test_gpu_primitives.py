"""GPU parity of the primitive hot-path operations against the oracle.

Tolerances: FP64 path 1e-11 relative (max-norm), mixed path (complex64 FFTs
and H.psi) 2e-5 relative; integer tables bit-exact.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11
FP32_TOL = 2e-5


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def make_pair(oracle, L=7.0, ecut=6.0, nb=6, kpts=((0.1, 0.2, -0.3),), nelec=4.0, seed=0,
              precision=0, n_fine=None, cell=None):
    import derek_gb300 as dg
    rng = np.random.default_rng(seed)
    wells = oracle.random_wells(rng, 3)
    cell = np.eye(3) * L if cell is None else np.asarray(cell, dtype=float)
    n_std, nf = oracle.grid_sizes(cell, ecut, 2.0, "smooth23")
    if n_fine is not None:
        nf = tuple(n_fine)
    vext = oracle.vext_jellium_wells(cell, nf, nelec, wells)
    s = oracle.System(cell, ecut, nf, n_std, np.array(kpts, dtype=float),
                      np.full(len(kpts), 1.0 / len(kpts)), nb, nelec, 0.01, vext, wells)
    spec = dg.SystemSpec(cell, ecut, kpts, nb, nelec, kT=0.01, vext=vext, n_fine=nf,
                         inv_cell=oracle.inv_cell(cell))
    return s, spec


@pytest.mark.parametrize("n", [(32, 32, 32), (30, 30, 30), (65, 65, 65), (42, 42, 42), (72, 72, 72),
                               (24, 36, 30), (13, 11, 7)])
def test_fft3d_matches_numpy(oracle, n):
    import derek_gb300 as dg
    L = 10.0
    spec = dg.SystemSpec(np.eye(3) * L, 1.0, [[0, 0, 0]], 2, 2.0, n_fine=n)
    rng = np.random.default_rng(1)
    a = rng.standard_normal(np.prod(n)) + 1j * rng.standard_normal(np.prod(n))
    with dg.Handle(spec) as h:
        for d in (1, -1):
            got = h.fft_3d(a, d)
            ref = oracle.fft3d(a, n, d)
            assert rel_err(got, ref) < 1e-13, (n, d, rel_err(got, ref))


def test_gsphere_tables_bit_exact(oracle):
    import derek_gb300 as dg
    cell = np.eye(3) * 16.0
    ks = oracle.mp_kpoints((4, 4, 4))[:6]
    spec = dg.SystemSpec(cell, 20.0, ks, 2, 2.0, inv_cell=oracle.inv_cell(cell))
    with dg.Handle(spec) as h:
        nf, ns = h.grid()
        assert nf == (72, 72, 72) and ns == (33, 33, 33)
        for ik, k in enumerate(ks):
            rows, fidx, kin = h.gsphere(0, ik)
            r2, mil, kin2 = oracle.gsphere(cell, 20.0, k, ns, inv_cell_given=oracle.inv_cell(cell))
            assert np.array_equal(rows, r2)
            assert np.array_equal(fidx, oracle.fft_flat_index(mil, nf))
            assert np.array_equal(kin, kin2)


@pytest.mark.parametrize("precision,tol", [(0, FP64_TOL), (1, FP32_TOL)])
@pytest.mark.parametrize("geom", ["cubic", "reference_rule", "triclinic"])
def test_apply_h_matches_oracle(oracle, precision, tol, geom):
    import derek_gb300 as dg
    kw = {}
    if geom == "reference_rule":
        kw = dict(L=7.3, ecut=5.0, n_fine=oracle.grid_sizes(np.eye(3) * 7.3, 5.0, 2.0, "reference")[1])
    if geom == "triclinic":
        kw = dict(cell=np.array([[7.0, 0.4, 0.0], [0.0, 6.5, 0.3], [0.2, 0.0, 7.5]]), ecut=5.0)
    s, spec = make_pair(oracle, **kw)
    kb = oracle.KBasis(s, 0)
    rng = np.random.default_rng(5)
    psi = rng.standard_normal((s.nbands, kb.npw)) + 1j * rng.standard_normal((s.nbands, kb.npw))
    v = s.vext + 0.3 * rng.standard_normal(s.nr)
    with dg.Handle(spec, precision=precision) as h:
        h.set_vloc(v)
        h.set_wfn(psi)
        got = h.pot_apply_wfn()
    ref = oracle.apply_h(s, kb, v, psi)
    assert rel_err(got, ref) < tol


@pytest.mark.parametrize("precision,tol", [(0, FP64_TOL), (1, FP32_TOL)])
def test_density_matches_oracle(oracle, precision, tol):
    import derek_gb300 as dg
    kpts = [(0.0, 0.0, 0.0), (0.25, -0.25, 0.25), (-0.25, 0.25, 0.25)]
    s, spec = make_pair(oracle, kpts=kpts, nb=5)
    rng = np.random.default_rng(7)
    occ = rng.uniform(0, 2, (len(kpts), s.nbands))
    occ[1, 3] = 0.0
    ref = np.zeros(s.nr)
    with dg.Handle(spec, precision=precision) as h:
        for ik in range(len(kpts)):
            kb = oracle.KBasis(s, ik)
            psi = rng.standard_normal((s.nbands, kb.npw)) + 1j * rng.standard_normal((s.nbands, kb.npw))
            psi /= np.linalg.norm(psi, axis=1)[:, None]
            h.set_wfn(psi, 0, ik)
            ref += s.wk[ik] * oracle.band_density(s, kb, psi, occ[ik])
        got = h.density_calculate(occ)
    assert rel_err(got, ref) < tol
    # charge: integral of n equals sum_k w_k sum_b f (orthogonality not needed)
    assert abs(got.sum() * s.volume / s.nr - (s.wk[:, None] * occ).sum()) < 1e-9 * occ.sum() + tol


REG_LENGTHS = [24, 27, 32, 36, 48, 54, 64, 72]


def reg_plane_pair(oracle, n, rows, kpts, nb, seed):
    """Cubic cell on an n^3 grid whose sphere reaches max(|mx|, |my|, |mz|) =
    N/4 - 2 ("tight": from N = 48 on, kernels that keep only those x, y and z
    line positions), N/4 + 1 ("compact") or N/4 + 3 ("all": every position
    kept)."""
    L = 8.0
    rmax = {"tight": n // 4 - 2, "compact": n // 4 + 1, "all": n // 4 + 3}[rows]
    rho = rmax + 0.25   # Miller radius; k_y = 0.2 puts the extreme rows at +-rmax
    ecut = 0.5 * (rho * 2 * np.pi / L) ** 2
    s, spec = make_pair(oracle, L=L, ecut=ecut, nb=nb, kpts=kpts, seed=seed, n_fine=(n, n, n))
    mil = np.concatenate([oracle.KBasis(s, ik).miller for ik in range(len(kpts))])
    assert int(np.abs(mil).max()) == rmax
    return s, spec


@pytest.mark.parametrize("rows", ["tight", "compact", "all"])
@pytest.mark.parametrize("n", REG_LENGTHS)
def test_apply_h_register_planes(oracle, n, rows):
    """FP32 H.psi through the register-line plane kernels at every compiled
    length, against the FP64 oracle."""
    import derek_gb300 as dg
    s, spec = reg_plane_pair(oracle, n, rows, ((0.1, 0.2, -0.3),), 3, seed=n)
    kb = oracle.KBasis(s, 0)
    rng = np.random.default_rng(n + 1)
    psi = rng.standard_normal((s.nbands, kb.npw)) + 1j * rng.standard_normal((s.nbands, kb.npw))
    v = s.vext + 0.3 * rng.standard_normal(s.nr)
    with dg.Handle(spec, precision=1) as h:
        h.set_vloc(v)
        h.set_wfn(psi)
        got = h.pot_apply_wfn()
    assert rel_err(got, oracle.apply_h(s, kb, v, psi)) < FP32_TOL


@pytest.mark.parametrize("rows", ["tight", "compact", "all"])
@pytest.mark.parametrize("n", REG_LENGTHS)
def test_density_register_planes(oracle, n, rows):
    """FP32 density through the register-line plane kernels (band loop with
    FP32 partial sums flushed to FP64), against the FP64 oracle."""
    import derek_gb300 as dg
    kpts = [(0.1, 0.2, -0.3), (-0.25, 0.2, 0.25)]
    nb = 11   # more bands than one flush period
    s, spec = reg_plane_pair(oracle, n, rows, kpts, nb, seed=2 * n)
    rng = np.random.default_rng(n + 3)
    occ = rng.uniform(0, 2, (len(kpts), nb))
    occ[0, 4] = 0.0
    ref = np.zeros(s.nr)
    with dg.Handle(spec, precision=1) as h:
        for ik in range(len(kpts)):
            kb = oracle.KBasis(s, ik)
            psi = rng.standard_normal((nb, kb.npw)) + 1j * rng.standard_normal((nb, kb.npw))
            psi /= np.linalg.norm(psi, axis=1)[:, None]
            h.set_wfn(psi, 0, ik)
            ref += s.wk[ik] * oracle.band_density(s, kb, psi, occ[ik])
        got = h.density_calculate(occ)
    assert rel_err(got, ref) < FP32_TOL


def test_xc_lda_matches_oracle_and_libxc(oracle):
    import derek_gb300 as dg
    spec = dg.SystemSpec(np.eye(3) * 6.0, 2.0, [[0, 0, 0]], 2, 2.0, n_fine=(8, 8, 8))
    rng = np.random.default_rng(2)
    rho = np.concatenate([10 ** rng.uniform(-14, 3, 5000), [0.0, 1e-15, 2e-15, 1e-16, -1.0]])
    with dg.Handle(spec) as h:
        exc, vxc = h.xc_lda(rho)
        e_ref, v_ref = oracle.lda_exc_vxc(rho)
        # PW92 evaluates log(1 + 1/q1) like libxc; for n < 1e-8 the argument is
        # within 1e-4 of 1 and a one-ulp difference in q1 is amplified, so the
        # tolerance is looser there
        big = rho >= 1e-8
        assert np.allclose(exc[big], e_ref[big], rtol=1e-13, atol=0)
        assert np.allclose(vxc[big], v_ref[big], rtol=1e-13, atol=0)
        assert np.allclose(exc, e_ref, rtol=1e-8, atol=0)
        assert np.allclose(vxc, v_ref, rtol=1e-8, atol=0)
        with open(os.path.join(os.path.dirname(__file__), "golden", "libxc_lda_unpol.json")) as f:
            data = json.load(f)["systems"]
        for d in data.values():
            r = np.array(d["rho"])
            e, v = h.xc_lda(r)
            ge = np.array(d["zk_x"]) + np.array(d["zk_c"])
            gv = np.array(d["vrho_x"]) + np.array(d["vrho_c"])
            assert np.allclose(e, ge, rtol=1e-12, atol=0)
            assert np.allclose(v, gv, rtol=1e-12, atol=0)


def test_uneven_batch_apply_h(oracle):
    """Two systems of different grids and sphere sizes in one handle."""
    import derek_gb300 as dg
    s1, sp1 = make_pair(oracle, L=6.0, ecut=5.0, nb=4, seed=1)
    s2, sp2 = make_pair(oracle, L=8.5, ecut=6.0, nb=7, seed=2, kpts=((0.0, 0.0, 0.0), (0.5, 0.5, 0.0)))
    rng = np.random.default_rng(9)
    with dg.Handle([sp1, sp2]) as h:
        for si, s in enumerate((s1, s2)):
            v = s.vext + 0.2 * rng.standard_normal(s.nr)
            h.set_vloc(v, si)
            for ik in range(len(s.kpts)):
                kb = oracle.KBasis(s, ik)
                psi = rng.standard_normal((s.nbands, kb.npw)) + 1j * rng.standard_normal((s.nbands, kb.npw))
                h.set_wfn(psi, si, ik)
                got = h.pot_apply_wfn(si, ik)
                assert rel_err(got, oracle.apply_h(s, kb, v, psi)) < FP64_TOL


@pytest.mark.parametrize("nb", [6, 20, 88])
def test_overlap_tensor_cores_match_fp64(oracle, nb):
    """S = psi^H psi of complex64 wavefunctions: split-BF16 tcgen05 path and
    the FP32 CUDA-core path against FP64 numpy on the same (FP32-rounded)
    data.  Tolerance relative to max|S|: 5e-5 for the tensor cores (the lo
    part of each operand is itself rounded to bf16, ~2^-17 per product, and
    the tensor-core FP32 accumulation of a 2048-coefficient split adds to
    it), 5e-6 for FP32 (single-precision sums over npw ~ 1000 terms;
    measured 1.6e-6)."""
    import derek_gb300 as dg
    L = 9.0 if nb < 50 else 12.0
    s, spec = make_pair(oracle, L=L, ecut=6.0, nb=nb, nelec=2.0)
    kb = oracle.KBasis(s, 0)
    rng = np.random.default_rng(nb)
    psi = rng.standard_normal((nb, kb.npw)) + 1j * rng.standard_normal((nb, kb.npw))
    psi32 = psi.astype(np.complex64).astype(np.complex128)
    ref = psi32.conj() @ psi32.T
    for tc, tol in ((1, 5e-5), (0, 5e-6)):
        with dg.Handle(spec, precision=1, use_tensor_cores=tc, buffer_bands=0) as h:
            h.set_wfn(psi)
            got = h.wave_dot()
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err < tol, (tc, err)
