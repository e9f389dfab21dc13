"""ctypes declarations of the C ABI in include/qpad_gpu.h.

The shared library is built in-tree by ``qpad_gb300.build`` (nvcc, sm_103a).  There is no
fallback: if the library is missing or cannot be loaded, importing the product raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

D = C.POINTER(C.c_double)
F = C.POINTER(C.c_float)
I32P = C.POINTER(C.c_int32)
I64P = C.POINTER(C.c_int64)


class GridDesc(C.Structure):
    _fields_ = [("nr", C.c_int32), ("nz", C.c_int32), ("max_mode", C.c_int32), ("bnd", C.c_int32),
                ("dr", C.c_double), ("dxi", C.c_double), ("relax_fac", C.c_double),
                ("iter_max", C.c_int32), ("iter_reltol", C.c_double), ("iter_abstol", C.c_double),
                ("dt", C.c_double), ("precision", C.c_int32), ("device", C.c_int32)]


class SpeciesDesc(C.Structure):
    _fields_ = [("qbm", C.c_double), ("push_type", C.c_int32), ("neutralized", C.c_int32),
                ("npmax", C.c_int64), ("sort_freq", C.c_int32)]


class BeamDesc(C.Structure):
    _fields_ = [("qbm", C.c_double), ("push_type", C.c_int32), ("evolution", C.c_int32),
                ("npmax", C.c_int64)]


class SliceStats(C.Structure):
    _fields_ = [("iters", C.c_int32), ("rel_res", C.c_double), ("abs_res", C.c_double)]


class TuneResult(C.Structure):
    _fields_ = [("iter_cluster", C.c_int32), ("iter_us", C.c_double), ("item_ppl", C.c_int32),
                ("deposit_us", C.c_double)]


class BatchTuneResult(C.Structure):
    _fields_ = [("policy", C.c_int32), ("unroll", C.c_int32), ("step_ms", C.c_double)]


class LaserDesc(C.Structure):
    _fields_ = [("k0", C.c_double), ("iter", C.c_int32)]


class NeutralDesc(C.Structure):
    _fields_ = [("qm", C.c_double), ("qbm", C.c_double), ("push_type", C.c_int32), ("levels", C.c_int32),
                ("adk", D), ("wp", C.c_double), ("density", C.c_double), ("ppc1", C.c_int32),
                ("ppc2", C.c_int32), ("num_theta", C.c_int32), ("npmax", C.c_int64)]


class H5GridInfo(C.Structure):
    _fields_ = [("time", C.c_double), ("iter", C.c_int32), ("dt", C.c_double), ("timeunit", C.c_char_p),
                ("units", C.c_char_p), ("label", C.c_char_p), ("axis_min", C.c_double * 2),
                ("axis_max", C.c_double * 2), ("axis_name", C.c_char_p * 2), ("axis_label", C.c_char_p * 2),
                ("axis_units", C.c_char_p * 2), ("type", C.c_char_p)]


class Rng(C.Structure):
    _fields_ = [("s", C.c_uint64), ("have", C.c_int32), ("next", C.c_double)]


class BeamLoadDesc(C.Structure):
    _fields_ = [("tot_num", C.c_int64), ("tot_charge", C.c_double), ("qm", C.c_double),
                ("gamma", C.c_double), ("center", C.c_double * 3), ("sigma", C.c_double * 3),
                ("range_lo", C.c_double * 3), ("range_hi", C.c_double * 3),
                ("uth", C.c_double * 3), ("quiet", C.c_int32)]


# status codes and enums (qpad_gpu.h)
OK, E_ARG, E_CUDA, E_NOMEM, E_CAPACITY, E_STATE = range(6)
BND_ZERO, BND_OPEN = 2, 3
PUSH2_STD, PUSH2_ROBUST = 0, 1
PUSH2_STD_PGC, PUSH2_ROBUST_PGC = 4, 5
PUSH3_REDUCED, PUSH3_BORIS = 1, 2
COPY_1TO2, COPY_2TO1 = 1, -1
PREC_FP64, PREC_MIXED = 0, 1
FIELDS = ["psi", "e", "e_spe", "b", "b_spe", "b_beam", "cu", "amu", "acu", "dcu", "q_spe", "q_beam"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}
FIELD_NCOMP = {"psi": 1, "e": 3, "e_spe": 3, "b": 3, "b_spe": 3, "b_beam": 3, "cu": 3, "amu": 3,
               "acu": 2, "dcu": 2, "q_spe": 1, "q_beam": 1}

_SIGS = {
    "qpad_ctx_create": (C.c_int, [C.POINTER(GridDesc), C.POINTER(C.c_void_p)]),
    "qpad_ctx_destroy": (C.c_int, [C.c_void_p]),
    "qpad_last_error": (C.c_char_p, [C.c_void_p]),
    "qpad_synchronize": (C.c_int, [C.c_void_p]),
    "qpad_field_layout": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), I64P]),
    "qpad_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "qpad_launch_count": (C.c_int, [C.c_void_p, I64P]),
    "qpad_set_graph": (C.c_int, [C.c_void_p, C.c_int]),
    "qpad_set_smooth": (C.c_int, [C.c_void_p, C.c_int]),
    "qpad_graph_active": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "qpad_graph_status": (C.c_char_p, [C.c_void_p]),
    "qpad_profile_enable": (C.c_int, [C.c_void_p, C.c_int]),
    "qpad_profile_read": (C.c_int, [C.c_void_p, C.c_char_p, D, I64P]),
    "qpad_species_reset": (C.c_int, [C.c_void_p]),
    "qpad_field_upload": (C.c_int, [C.c_void_p, C.c_int, C.c_int, D]),
    "qpad_field_download": (C.c_int, [C.c_void_p, C.c_int, C.c_int, D]),
    "qpad_store_download": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, D]),
    "qpad_store_read": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, D]),
    "qpad_store_upload": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, D]),
    "qpad_field_fill": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "qpad_store_fill": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "qpad_field_add": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "qpad_field_add_dim": (C.c_int, [C.c_void_p, C.c_int, C.c_int, I32P, I32P, C.c_int]),
    "qpad_field_scale": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "qpad_field_copy_slice": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "qpad_solve_psi": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qpad_solve_bz": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qpad_solve_bt_beam": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qpad_solve_bt_iter": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "qpad_solve_ez": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qpad_solve_et": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "qpad_solve_djdxi": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "qpad_conv_test": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, D, D]),
    "qpad_species_create": (C.c_int, [C.c_void_p, C.POINTER(SpeciesDesc), D, D, D, D, D, C.c_int64,
                                      C.POINTER(C.c_void_p)]),
    "qpad_species_destroy": (C.c_int, [C.c_void_p]),
    "qpad_species_renew": (C.c_int, [C.c_void_p, D, D, D, D, D, C.c_int64]),
    "qpad_species_download": (C.c_int, [C.c_void_p, D, D, D, D, D, I64P]),
    "qpad_species_count": (C.c_int, [C.c_void_p, I64P]),
    "qpad_species_qdp": (C.c_int, [C.c_void_p, C.c_int]),
    "qpad_species_cbq": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "qpad_species_amjdp": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]),
    "qpad_species_amjdp_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.c_double]),
    "qpad_species_push_u": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_double]),
    "qpad_species_push_x": (C.c_int, [C.c_void_p, C.c_double]),
    "qpad_species_interp_psi": (C.c_int, [C.c_void_p, C.c_int]),
    "qpad_species_sort": (C.c_int, [C.c_void_p]),
    "qpad_beam_create": (C.c_int, [C.c_void_p, C.POINTER(BeamDesc), D, D, D, C.c_int64, C.POINTER(C.c_void_p)]),
    "qpad_beam_destroy": (C.c_int, [C.c_void_p]),
    "qpad_beam_download": (C.c_int, [C.c_void_p, D, D, D, I64P]),
    "qpad_beam_count": (C.c_int, [C.c_void_p, I64P]),
    "qpad_beam_qdp": (C.c_int, [C.c_void_p, C.c_int]),
    "qpad_beam_push": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qpad_slice_step": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(SliceStats)]),
    "qpad_3d_step": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(SliceStats)]),
    "qpad_learn_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int,
                                    C.POINTER(C.c_void_p)]),
    "qpad_learn_destroy": (C.c_int, [C.c_void_p]),
    "qpad_learn_last_error": (C.c_char_p, [C.c_void_p]),
    "qpad_learn_param_count": (C.c_int, [C.c_void_p, I64P]),
    "qpad_learn_get_params": (C.c_int, [C.c_void_p, F]),
    "qpad_learn_set_params": (C.c_int, [C.c_void_p, F]),
    "qpad_learn_predict": (C.c_int, [C.c_void_p, F, C.c_int64, C.c_int, F]),
    "qpad_learn_grad": (C.c_int, [C.c_void_p, F, F, C.c_int64, C.c_int, D, F]),
    "qpad_learn_train": (C.c_int, [C.c_void_p, F, F, C.c_int64, C.c_int, C.c_int, C.c_int, C.c_float,
                                   C.c_uint64, D]),
    "qpad_guess_attach": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "qpad_guess_sample": (C.c_int, [C.c_void_p, C.c_int, C.c_int, F, F, F]),
    "qpad_h5_last_error": (C.c_char_p, []),
    "qpad_neutral_create": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "qpad_neutral_state_download": (C.c_int, [C.c_void_p, D]),
    "qpad_laser_create": (C.c_int, [C.c_void_p, C.c_void_p, D, D, C.POINTER(C.c_void_p)]),
    "qpad_laser_download": (C.c_int, [C.c_void_p, D, D]),
    "qpad_laser_chi_download": (C.c_int, [C.c_void_p, D]),
    "qpad_lasers_advance": (C.c_int, [C.c_void_p]),
    "qpad_set_launch_shapes": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "qpad_set_graph_unroll": (C.c_int, [C.c_void_p, C.c_int]),
    "qpad_guess_apply": (C.c_int, [C.c_void_p, C.c_int]),
    "qpad_species_set_radial_ppc": (C.c_int, [C.c_void_p, C.c_int32]),
    "qpad_h5_write_grid": (C.c_int, [C.c_char_p, C.c_char_p, D, C.c_int, C.c_int, C.c_void_p]),
    "qpad_h5_write_particles": (C.c_int, [C.c_char_p, C.c_char_p, D, D, D, C.c_int64, C.c_int, C.c_double,
                                          C.c_double]),
    "qpad_h5_read_dataset": (C.c_int, [C.c_char_p, C.c_char_p, D, C.c_int64, I64P, I32P, I64P]),
    "qpad_h5_read_attr": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, D, C.c_char_p, C.c_int64]),
    "qpad_diag_write_field": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_char_p, C.c_char_p, C.c_char_p,
                                        C.c_char_p, C.c_int, C.c_double, C.c_double]),
    "qpad_beam_write_rst": (C.c_int, [C.c_void_p, C.c_char_p, C.c_char_p, C.c_int, C.c_double, C.c_double]),
    "qpad_rst_read": (C.c_int, [C.c_char_p, D, D, D, C.c_int64, I64P]),
    "qpad_set_guess_extrapolation": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "qpad_guess_samples": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, F, F, F]),
    "qpad_guess_config": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "qpad_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.POINTER(C.c_void_p)]),
    "qpad_batch_destroy": (C.c_int, [C.c_void_p]),
    "qpad_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "qpad_batch_step": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.POINTER(SliceStats))]),
    "qpad_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(TuneResult)]),
    "qpad_batch_autotune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(BatchTuneResult)]),
    "qpad_rng_seed": (None, [C.POINTER(Rng), C.c_uint64]),
    "qpad_load_plasma": (C.c_int64, [C.c_int, C.c_double, C.POINTER(Rng), C.c_int, C.c_int, C.c_int, C.c_double,
                                     C.c_double, D, D, D, D, D, D, C.c_int64]),
    "qpad_load_beam": (C.c_int64, [C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(Rng),
                                   C.POINTER(BeamLoadDesc), D, D, D, C.c_int64]),
}

EXPORTED = sorted(_SIGS)

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libqpad_gpu.so (building it first if absent); raises if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; run qpad_gb300.build.build()")
        _build.build()
    L = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L
