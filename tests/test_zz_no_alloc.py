"""The overlap entry point that allocates nothing (derek_gpu_overlap_noalloc).

Callers that cannot call cudaMalloc -- a host code that owns the device
memory pool, or one that forbids allocation after its set-up -- pass device
pointers for the wavefunctions and the result; the split-K scratch lives in a
file-scope device array inside the library.  This test calls it through the
C ABI twice in a row, with different inputs, and checks each result against
the handle path's derek_gpu_overlap on the same wavefunctions (1e-11
relative in FP64, the tolerance of the other FP64 parity tests).  The device
buffers are the test's own (allocated by torch), as such a caller's would be.
It runs alone in a fresh process or after the other tests; pytest collects
this file last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_overlap_noalloc_matches_handle_overlap(oracle):
    import torch
    import derek_gb300 as dg

    cell = np.eye(3) * 8.0
    ecut, nb = 6.0, 12
    n_std, nf = oracle.grid_sizes(cell, ecut, 2.0, "smooth23")
    spec = dg.SystemSpec(cell, ecut, [[0.1, -0.2, 0.3]], nb, 2.0, kT=0.01, n_fine=nf,
                         inv_cell=oracle.inv_cell(cell))
    rng = np.random.default_rng(11)
    with dg.Handle(spec, precision=dg.DEREK_PREC_FP64, buffer_bands=0) as h:
        npw = h.npw()
        for call in range(2):
            psi = rng.standard_normal((nb, npw)) + 1j * rng.standard_normal((nb, npw))
            h.set_wfn(psi)
            ref = h.wave_dot()
            x = torch.from_numpy(psi.view(np.float64).copy()).cuda()
            s = torch.zeros((nb, nb, 2), dtype=torch.float64, device="cuda")
            stream = torch.cuda.current_stream().cuda_stream
            st = dg.lib.derek_gpu_overlap_noalloc(
                ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()), nb, npw,
                ctypes.c_long(npw), dg.DEREK_PREC_FP64, ctypes.c_void_p(s.data_ptr()),
                ctypes.c_void_p(stream))
            assert st == 0, dg.lib.derek_gpu_strerror(st)
            torch.cuda.synchronize()
            got = s.cpu().numpy().view(np.complex128).reshape(nb, nb)
            err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
            assert err < 1e-11, (call, err)


def _noalloc(dg, x, y, nb, npw, ld, precision, s, stream):
    return dg.lib.derek_gpu_overlap_noalloc(
        ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), nb, npw, ctypes.c_long(ld),
        precision, ctypes.c_void_p(s.data_ptr()), ctypes.c_void_p(stream))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_overlap_noalloc_several_splits_padded_rows(oracle, precision):
    """npw = 11,000+ plane waves (three 4096-coefficient K-splits, so the
    reduction sums several partials), distinct X and Y (S is not Hermitian,
    so a swapped or wrongly conjugated operand fails), rows padded to
    ld = npw + 40 with garbage in the padding, two calls in a row.  Checked
    against FP64 numpy conj(X) @ Y.T: 1e-11 relative in FP64; complex64
    inputs against the same product of the rounded inputs, 1e-5 relative."""
    import torch
    import derek_gb300 as dg

    cell = np.eye(3) * 16.0
    n_std, nf = oracle.grid_sizes(cell, 15.0, 2.0, "smooth23")
    kb = oracle.KBasis(oracle.make_system(16.0, 15.0, 2.0, 4, np.zeros((0, 5)), kpts=[[0.1, 0.2, 0.3]]), 0)
    npw, nb = kb.npw, 40
    assert npw > 2 * 4096
    ld = npw + 40
    rng = np.random.default_rng(21)
    fp64 = precision == "fp64"
    prec = dg.DEREK_PREC_FP64 if fp64 else dg.DEREK_PREC_MIXED
    cdt = np.complex128 if fp64 else np.complex64
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        X = (rng.standard_normal((nb, ld)) + 1j * rng.standard_normal((nb, ld))).astype(cdt)
        Y = (rng.standard_normal((nb, ld)) + 1j * rng.standard_normal((nb, ld))).astype(cdt)
        X[:, npw:] = 1e30 if fp64 else 1e20
        Y[:, npw:] = np.nan
        real = np.float64 if fp64 else np.float32
        x = torch.from_numpy(X.view(real).copy()).cuda()
        y = torch.from_numpy(Y.view(real).copy()).cuda()
        s = torch.full((nb, nb, 2), np.nan, dtype=torch.float64, device="cuda")
        assert _noalloc(dg, x, y, nb, npw, ld, prec, s, stream) == 0
        torch.cuda.synchronize()
        got = s.cpu().numpy().view(np.complex128).reshape(nb, nb)
        Xd = X[:, :npw].astype(np.complex128)
        Yd = Y[:, :npw].astype(np.complex128)
        ref = Xd.conj() @ Yd.T
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err < (1e-11 if fp64 else 1e-5), (call, err)
        assert not np.allclose(ref, ref.conj().T)   # distinct operands: S is not Hermitian


def test_overlap_noalloc_rejects_sizes_beyond_its_scratch():
    import derek_gb300 as dg
    # nb above 128 or npw above 16 x 4096 exceeds the file-scope scratch array;
    # the arguments are rejected before any pointer is used
    st = dg.lib.derek_gpu_overlap_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 129, 100,
                                          ctypes.c_long(100), dg.DEREK_PREC_FP64,
                                          ctypes.c_void_p(16), None)
    assert st == dg._abi.DEREK_ERR_UNSUPPORTED
    st = dg.lib.derek_gpu_overlap_noalloc(ctypes.c_void_p(16), ctypes.c_void_p(16), 8, 70000,
                                          ctypes.c_long(70000), dg.DEREK_PREC_FP64,
                                          ctypes.c_void_p(16), None)
    assert st == dg._abi.DEREK_ERR_UNSUPPORTED
