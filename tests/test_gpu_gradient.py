"""Hellmann-Feynman gradient of the converged free energy with respect to the
Gaussian-well parameters, checked against central finite differences of the
FP64 GPU SCF (h = 1e-4; tolerance 2e-6 Ha per unit parameter), and the
depth derivative against the analytic identity dF/dU_w = -int n e_w."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_energy(dg, cell, kpts, wells, nb=6, nelec=4.0):
    spec = dg.SystemSpec(cell, 6.0, kpts, nb, nelec, kT=0.01, wells=wells)
    with dg.Handle(spec, precision=dg.DEREK_PREC_FP64, density_tol=1e-10) as h:
        rep = h.electronic_scf(max_scf=300, etol=1e-13)[0]
        g = h.grad_wells()
        rho = h.density()
        nf, _ = h.grid()
    return rep["free_energy"], g, rho, nf


def test_hellmann_feynman_matches_finite_differences(oracle):
    import derek_gb300 as dg
    cell = np.eye(3) * 7.0
    kpts = [[0.0, 0.0, 0.0], [0.25, 0.25, 0.25]]
    rng = np.random.default_rng(4)
    wells = oracle.random_wells(rng, 3)
    F0, g, rho, nf = _free_energy(dg, cell, kpts, wells)
    assert g.shape == (3, 5)
    h = 1e-4
    for (w, p) in ((0, 3), (1, 4), (2, 0), (0, 2)):
        wp = wells.copy()
        wm = wells.copy()
        wp[w, p] += h
        wm[w, p] -= h
        Fp = _free_energy(dg, cell, kpts, wp)[0]
        Fm = _free_energy(dg, cell, kpts, wm)[0]
        fd = (Fp - Fm) / (2 * h)
        assert abs(fd - g[w, p]) < 2e-6, (w, p, fd, g[w, p])
    # dF/dU_w = -int n(r) exp(-|r - R_w|^2 / (2 s_w^2)) dr on the same grid
    frac = oracle.real_frac_points(nf)
    for w in range(3):
        d = frac - wells[w, :3][None, :]
        d -= np.rint(d)
        r2 = ((d @ cell.T) ** 2).sum(1)
        e = np.exp(-r2 / (2 * wells[w, 4] ** 2))
        ref = -np.sum(rho * e) * np.linalg.det(cell) / rho.size
        assert abs(ref - g[w, 3]) < 1e-10 * max(1.0, abs(ref))


def test_adjoint_density_loss_gradient_matches_finite_differences(oracle):
    """dL/dp of L = sum (n - n_target)^2 dV through the converged SCF (adjoint
    linear response) against central differences of L from full FP64 SCF runs
    (h = 1e-4); n_target comes from a second seeded well set."""
    import derek_gb300 as dg
    cell = np.eye(3) * 7.0
    kpts = [[0.0, 0.0, 0.0], [0.25, 0.25, 0.25]]
    rng = np.random.default_rng(4)
    wells = oracle.random_wells(rng, 3)
    target_wells = oracle.random_wells(np.random.default_rng(5), 3)
    _, _, n_t, _ = _free_energy(dg, cell, kpts, target_wells)

    def loss_and_grad(w, want_grad):
        spec = dg.SystemSpec(cell, 6.0, kpts, 6, 4.0, kT=0.01, wells=w)
        with dg.Handle(spec, precision=dg.DEREK_PREC_FP64, density_tol=1e-11) as h:
            h.electronic_scf(max_scf=400, etol=1e-14)
            if want_grad:
                return h.grad_density_loss(n_t, tol=1e-10)
            rho = h.density()
            return float(np.sum((rho - n_t) ** 2) * np.linalg.det(cell) / rho.size), None

    L0, g = loss_and_grad(wells, True)
    assert L0 > 0
    h = 1e-4
    for (w, p) in ((0, 3), (1, 4), (2, 1)):
        wp = wells.copy()
        wm = wells.copy()
        wp[w, p] += h
        wm[w, p] -= h
        fd = (loss_and_grad(wp, False)[0] - loss_and_grad(wm, False)[0]) / (2 * h)
        assert abs(fd - g[w, p]) < 1e-4 * max(1.0, abs(fd)), (w, p, fd, g[w, p])


def test_adjoint_config4_matches_oracle_finite_differences():
    """The adjoint-gradient workload (L=12 bohr, Ecut 15 Ha, 48^3 grid, Gamma
    + 2x2x2 k-points, 16 electrons in 20 bands, 8 wells): dL/dp of
    L = sum (n - n_target)^2 dV from the adjoint solve, and the
    Hellmann-Feynman dF/dp, against central differences (h = 1e-5) of the FP64
    oracle's converged SCFs for three parameters (a depth, a width, a centre
    coordinate; tests/golden/make_adjoint_golden.py).  n_target is the GPU's
    own FP64 ground state of the second well set, which equals the oracle's
    to the SCF tolerance.

    Tolerances, from measurement: the adjoint within 1e-6 (measured 2e-8 to
    3e-8, 3e-7 relative at most), Hellmann-Feynman within 1e-6 relative
    (measured 1.5e-9), and the GPU's own central difference of L for the
    centre coordinate within 1e-6 relative of the oracle's (measured 3.5e-8),
    which pins the two SCFs' loss to each other."""
    import os
    import derek_gb300 as dg
    from derek_gb300 import workloads
    d = dict(np.load(os.path.join(os.path.dirname(__file__), "golden", "adjoint9k.npz")))
    systems, mix = workloads.params("adjoint9k")
    assert np.array_equal(systems[0]["wells"], d["wells"])
    tgt = dict(systems[0], wells=d["target_wells"])
    opts = dict(mix, density_tol=1e-11)
    with dg.Handle(workloads.to_specs([tgt]), precision=dg.DEREK_PREC_FP64, **opts) as h:
        rt = h.electronic_scf(max_scf=400, etol=1e-13)[0]
        n_t = h.density()
    assert rt["converged"] and abs(rt["free_energy"] - d["target_free_energy"]) < 1e-8
    with dg.Handle(workloads.to_specs(systems), precision=dg.DEREK_PREC_FP64, **opts) as h:
        r0 = h.electronic_scf(max_scf=400, etol=1e-13)[0]
        hf = h.grad_wells()
        loss, g = h.grad_density_loss(n_t, tol=1e-11)
        dvol = abs(float(np.linalg.det(np.asarray(systems[0]["cell"])))) / n_t.size
    assert r0["converged"] and abs(r0["free_energy"] - d["free_energy"]) < 1e-8
    assert abs(loss - d["loss"]) < 1e-8 * max(1.0, abs(float(d["loss"])))
    for (w, c), fd_l, fd_f in zip(d["params"], d["fd_loss"], d["fd_free"]):
        assert abs(hf[w, c] - fd_f) < 1e-6 * max(1.0, abs(fd_f)), (w, c, hf[w, c], fd_f)
        assert abs(g[w, c] - fd_l) < 1e-6 * max(1.0, abs(fd_l)), (w, c, g[w, c], fd_l)
    # the GPU's own central difference of L for the centre coordinate
    (w, c), hstep = d["params"][2], float(d["h"])
    losses = []
    for sg in (1, -1):
        wl = systems[0]["wells"].copy()
        wl[w, c] += sg * hstep
        with dg.Handle(workloads.to_specs([dict(systems[0], wells=wl)]), precision=dg.DEREK_PREC_FP64,
                       **dict(mix, density_tol=1e-12)) as h:
            r = h.electronic_scf(max_scf=400, etol=1e-14)[0]
            assert r["converged"]
            losses.append(float(np.sum((h.density() - n_t) ** 2)) * dvol)
    fd_gpu = (losses[0] - losses[1]) / (2 * hstep)
    assert abs(fd_gpu - d["fd_loss"][2]) < 1e-6 * abs(d["fd_loss"][2]), (fd_gpu, d["fd_loss"][2])