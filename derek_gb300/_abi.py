"""ctypes declarations of include/derek_gpu.h and the library loader.

Loading is strict: a missing or unloadable ``libderek_gpu.so`` raises
ImportError -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os

DEREK_OK = 0
DEREK_ERR_BAD_ARG = 1
DEREK_ERR_OOM = 2
DEREK_ERR_CUDA = 3
DEREK_ERR_NOT_CONVERGED = 4
DEREK_ERR_CHOLESKY = 5
DEREK_ERR_NAN = 6
DEREK_ERR_TIMEOUT = 7
DEREK_ERR_UNSUPPORTED = 8

DEREK_TUNE_RETUNE = 1
DEREK_PREC_FP64 = 0
DEREK_PREC_MIXED = 1
DEREK_GRID_REFERENCE = 0
DEREK_GRID_SMOOTH23 = 1


class DerekError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


_d = ctypes.c_double
_i = ctypes.c_int
_pd = ctypes.POINTER(ctypes.c_double)


class SysDesc(ctypes.Structure):
    _fields_ = [
        ("cell", _d * 9), ("inv_cell", _d * 9), ("ecut", _d), ("g_fine_scale", _d),
        ("n_fine", _i * 3), ("grid_policy", _i), ("nk", _i), ("kpts", _pd), ("wk", _pd),
        ("nbands", _i), ("nspinor", _i), ("nelec", _d), ("kT", _d), ("vext", _pd),
        ("nwells", _i), ("wells", _pd),
    ]


_c32 = ctypes.c_char * 32


class InfoParams(ctypes.Structure):
    """derek_info (include/derek_gpu.h)."""
    _fields_ = (
        [(n, _i) for n in ("check", "debugging", "n_electrons", "max_scf", "conduction_bands", "nbands",
                           "iprint", "random_seed", "write_wvfn", "soc", "write_density", "write_potential",
                           "write_state", "write_spec", "write_memory", "write_formatted_potential",
                           "write_potex", "write_formatted_density", "restart", "write_formatted_potex",
                           "write_xsf")]
        + [(n, _i * 3) for n in ("kpt_mp_grid", "periodic_pot_grid", "dos_kpt_mp_grid")]
        + [(n, _d) for n in ("energy_tol", "cut_off_energy", "g_fine_scale", "electronic_temp",
                             "finite_barrier_height")]
        + [("finite_barrier_width", _d * 3), ("periodic_pot_amp", _d), ("ext_efield", _d * 3),
           ("ext_bfield", _d * 3)]
        + [(n, _c32) for n in ("xc_functional", "task", "scf_method", "external_pot", "output_level",
                               "unit_energy", "unit_length", "unit_efield", "unit_bfield", "out_energy_unit",
                               "out_len_unit", "out_efield_unit", "out_bfield_unit")]
        + [("cell", _d * 9), ("n_pots", _i), ("pot_centres", _d * 192), ("pot_heights", _d * 64),
           ("pot_widths", _d * 64), ("n_corrected", _i)]
    )


class ScfOpts(ctypes.Structure):
    _fields_ = [
        ("precision", _i), ("mix_alpha", _d), ("kerker_q0", _d), ("pulay_history", _i),
        ("cheb_degree", _i), ("first_passes", _i), ("first_degree", _i),
        ("seed", ctypes.c_uint64), ("use_graph", _i), ("use_tensor_cores", _i),
        ("density_tol", _d), ("buffer_bands", _i), ("etol_per_electron", _i),
        ("init_vectors", _i),
    ]


class ScfReport(ctypes.Structure):
    _fields_ = [
        ("energy", _d), ("free_energy", _d), ("delta", _d), ("efermi", _d), ("entropy", _d),
        ("e_band", _d), ("e_hartree", _d), ("e_xc", _d), ("e_dc", _d),
        ("residual", _d), ("iterations", _i), ("converged", _i),
    ]


def report_dict(r: ScfReport) -> dict:
    return {name: getattr(r, name) for name, _ in ScfReport._fields_}


# name -> (restype, argtypes)
_vp = ctypes.c_void_p
SIGNATURES = {
    "derek_gpu_default_opts": (None, [ctypes.POINTER(ScfOpts)]),
    "derek_gpu_strerror": (ctypes.c_char_p, [_i]),
    "derek_gpu_last_error": (ctypes.c_char_p, [_vp]),
    "derek_gpu_create": (_i, [ctypes.POINTER(_vp), ctypes.POINTER(SysDesc), _i, ctypes.POINTER(ScfOpts)]),
    "derek_gpu_destroy": (_i, [_vp]),
    "derek_gpu_grid": (_i, [_vp, _i, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "derek_gpu_npw": (_i, [_vp, _i, _i, ctypes.POINTER(_i)]),
    "derek_gpu_bands": (_i, [_vp, _i, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "derek_gpu_gsphere": (_i, [_vp, _i, _i, _vp, _vp, _pd]),
    "derek_gpu_fft3d": (_i, [_vp, _i, _pd, _i]),
    "derek_gpu_set_vloc": (_i, [_vp, _i, _pd]),
    "derek_gpu_get_vloc": (_i, [_vp, _i, _pd]),
    "derek_gpu_set_wfn": (_i, [_vp, _i, _i, _pd]),
    "derek_gpu_get_wfn": (_i, [_vp, _i, _i, _pd]),
    "derek_gpu_apply_h": (_i, [_vp, _i, _i, _pd]),
    "derek_gpu_density": (_i, [_vp, _i, _pd, _pd]),
    "derek_gpu_density_spinor": (_i, [_vp, _i, _pd, _pd, _pd]),
    "derek_gpu_set_nc_pot": (_i, [_vp, _i, _pd]),
    "derek_gpu_get_nc_pot": (_i, [_vp, _i, _pd]),
    "derek_gpu_get_nc_ext": (_i, [_vp, _i, _pd]),
    "derek_gpu_get_magnetisation": (_i, [_vp, _i, _pd]),
    "derek_gpu_set_start_magnetisation": (_i, [_vp, _i, _pd]),
    "derek_gpu_xc_lsda": (_i, [_vp, ctypes.c_long, _pd, _pd, _pd, _pd, _pd]),
    "derek_gpu_xc_lda": (_i, [_vp, ctypes.c_long, _pd, _pd, _pd]),
    "derek_gpu_overlap": (_i, [_vp, _i, _i, _pd]),
    "derek_gpu_overlap_noalloc": (_i, [_vp, _vp, _i, _i, ctypes.c_long, _i, _vp, _vp]),
    "derek_gpu_scf_iterate": (_i, [_vp, ctypes.POINTER(ScfReport)]),
    "derek_gpu_scf_run": (_i, [_vp, _i, _d, ctypes.POINTER(ScfReport)]),
    "derek_gpu_grad_wells": (_i, [_vp, _i, _pd]),
    "derek_gpu_grad_density_loss": (_i, [_vp, _i, _pd, _pd, _pd, _i, _d]),
    "derek_gpu_get_eigenvalues": (_i, [_vp, _i, _pd]),
    "derek_gpu_get_occupations": (_i, [_vp, _i, _pd]),
    "derek_gpu_get_density": (_i, [_vp, _i, _pd]),
    "derek_gpu_set_vext": (_i, [_vp, _i, _pd]),
    "derek_gpu_get_vext": (_i, [_vp, _i, _pd]),
    "derek_gpu_stream": (_vp, [_vp]),
    "derek_gpu_launch_count": (ctypes.c_ulonglong, []),
    "derek_gpu_time_apply_h": (_i, [_vp, _i, _pd, _pd]),
    "derek_gpu_autotune": (_i, [_vp, ctypes.c_char_p, _i]),
    "derek_gpu_set_wait_limit": (_i, [ctypes.c_long]),
    "derek_gpu_plan": (_i, [_vp, ctypes.c_char_p, _i]),
    "derek_host_tune_cache_normalise": (_i, [ctypes.c_char_p, ctypes.c_char_p, _i]),
    "derek_host_radix_candidates": (_i, [_i, ctypes.c_char_p, _i]),
    "derek_gpu_set_start_density": (_i, [_vp, _i, _pd]),
    "derek_info_read": (_i, [ctypes.c_char_p, ctypes.POINTER(InfoParams), ctypes.c_char_p, _i]),
    "derek_gpu_nscf_run": (_i, [_vp, _i, _d, _i, ctypes.POINTER(_i)]),
    "derek_io_write_den": (_i, [ctypes.c_char_p, ctypes.POINTER(_i), ctypes.c_longlong, _pd, _pd]),
    "derek_io_read_den": (_i, [ctypes.c_char_p, ctypes.POINTER(_i), ctypes.c_longlong, _pd, _pd]),
    "derek_io_write_pot": (_i, [ctypes.c_char_p, ctypes.POINTER(_i), ctypes.c_longlong, _pd]),
    "derek_io_read_pot": (_i, [ctypes.c_char_p, ctypes.POINTER(_i), ctypes.c_longlong, _pd]),
    "derek_io_write_wvfn": (_i, [ctypes.c_char_p, ctypes.POINTER(_i), ctypes.c_longlong, _i, _i, _i, _pd]),
    "derek_io_read_wvfn": (_i, [ctypes.c_char_p, ctypes.POINTER(_i), ctypes.c_longlong, _i, _i, _i, _pd]),
    "derek_io_write_xsf": (_i, [ctypes.c_char_p, ctypes.POINTER(_d), ctypes.POINTER(_i), _pd]),
    "derek_io_write_fden": (_i, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), _pd, _pd]),
    "derek_io_write_fpot": (_i, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), _pd]),
    "derek_io_set_subrecord_limit": (_i, [ctypes.c_longlong]),
    "derek_host_prime_fact": (_i, [_i]),
    "derek_host_grid_sizes": (_i, [ctypes.POINTER(_d), _d, _d, _i, ctypes.POINTER(_i), ctypes.POINTER(_i)]),
    "derek_host_gsphere": (_i, [ctypes.POINTER(_d), _d, ctypes.POINTER(_d), ctypes.POINTER(_i), _i, _vp,
                                ctypes.POINTER(_i)]),
}

lib_path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libderek_gpu.so")


def _load():
    if not os.path.exists(lib_path):
        raise ImportError(f"{lib_path} is missing: run derek_gb300/build.py "
                          "(there is no CPU fallback for the GPU path)")
    L = ctypes.CDLL(lib_path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


lib = _load()
