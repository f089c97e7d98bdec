"""ctypes binding of libtnkit_gb300.so (include/tnkit_gb300.h).

The library is loaded from this package directory only. There is no fallback: if the library
is missing or fails to load, every compute call raises `LibraryMissing` -- the product never
silently runs a CPU or library path in its place.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtnkit_gb300.so")

TNK_OK, TNK_ERR_ARG, TNK_ERR_CUDA, TNK_ERR_SIZE, TNK_ERR_DEVICE = 0, 1, 2, 3, 4
TNK_RED_ELEMS = 65536
TNK_TRIDIAG_MAX_N = 128


class LibraryMissing(RuntimeError):
    pass


class TnkError(RuntimeError):
    """A nonzero status from the library, with its message."""

    def __init__(self, code, where, msg):
        super().__init__(f"{where}: status {code}: {msg}")
        self.code = code


# numpy mirrors of the table structs (sizes checked against tnk_struct_sizes at load)
GEMM_TASK = np.dtype([("c_off", "<i8"), ("ldc", "<i4"), ("m", "<i4"), ("n", "<i4"),
                      ("seg_begin", "<i4"), ("seg_end", "<i4"), ("flags", "<i4")])
GEMM_SEG = np.dtype([("a_off", "<i8"), ("b_off", "<i8"), ("a_rs", "<i4"), ("a_cs", "<i4"),
                     ("b_rs", "<i4"), ("b_cs", "<i4"), ("k", "<i4"), ("a_buf", "<i2"),
                     ("b_buf", "<i2"), ("conj", "<i4"), ("pad", "<i4"), ("coef", "<f8")])
GEMM_TILE = np.dtype([("task", "<i4"), ("m0", "<i4"), ("n0", "<i4"), ("pad", "<i4")])
GEBRD_SECTOR = np.dtype([("m", "<i8"), ("n", "<i8"), ("a_off", "<i8"), ("ul_off", "<i8"),
                         ("vr_off", "<i8"), ("v_off", "<i8"), ("spare", "<i8"), ("a_rs", "<i4"),
                         ("a_cs", "<i4")])
REFL_SET = np.dtype([("rows", "<i8"), ("nrefl", "<i8"), ("r_off", "<i8"), ("tau_off", "<i8"),
                     ("z_off", "<i8"), ("shift", "<i4"), ("pad", "<i4")])
COMB_TASK = np.dtype([("dst_off", "<i8"), ("rows", "<i4"), ("cols", "<i4"), ("dst_ld", "<i4"),
                      ("dst_cs", "<i4"), ("term_begin", "<i4"), ("term_end", "<i4")])
COMB_TERM = np.dtype([("src_off", "<i8"), ("src_ld", "<i4"), ("src_cs", "<i4"),
                      ("coef", "<f8")])
COMB_ITEM = np.dtype([("task", "<i4"), ("row0", "<i4"), ("row1", "<i4"), ("pad", "<i4")])
TC_SEG = np.dtype([("a_map", "<i4"), ("b_map", "<i4"), ("k", "<i4"), ("pad", "<i4")])
CVT_TASK = np.dtype([("src_off", "<i8"), ("dst_off", "<i8"), ("rows", "<i4"), ("cols", "<i4"),
                     ("src_ld", "<i4"), ("dst_ld", "<i4"), ("transpose", "<i4"), ("pad", "<i4")])
CVT_ITEM = np.dtype([("task", "<i4"), ("r0", "<i4"), ("c0", "<i4"), ("pad", "<i4")])


class LayoutDesc(C.Structure):
    _fields_ = [("nlegs", C.c_int32), ("nblocks", C.c_int32), ("keys", C.c_void_p),
                ("shapes", C.c_void_p), ("offsets", C.c_void_p)]


class ApplyPlanIn(C.Structure):
    _fields_ = [("n_sites", C.c_int32), ("pad", C.c_int32), ("theta", LayoutDesc),
                ("L", LayoutDesc), ("R", LayoutDesc), ("out", LayoutDesc), ("S", C.c_void_p),
                ("s_dims", C.c_int64 * 6), ("sec_start", C.c_void_p), ("sec_dim", C.c_void_p),
                ("sec_begin", C.c_int64 * 7)]


class EnvPlanIn(C.Structure):
    _fields_ = [("side", C.c_int32), ("pad", C.c_int32), ("env", LayoutDesc),
                ("site", LayoutDesc), ("out", LayoutDesc), ("W", C.c_void_p),
                ("w_dims", C.c_int64 * 4), ("sec_start", C.c_void_p), ("sec_dim", C.c_void_p),
                ("sec_begin", C.c_int64 * 5)]


class Plan3(C.Structure):
    _fields_ = [("t1", C.c_void_p), ("s1", C.c_void_p), ("tiles1", C.c_void_p),
                ("n_tiles1", C.c_int64),
                ("t2", C.c_void_p), ("c2", C.c_void_p), ("items2", C.c_void_p),
                ("n_items2", C.c_int64),
                ("t3", C.c_void_p), ("s3", C.c_void_p), ("tiles3", C.c_void_p),
                ("n_tiles3", C.c_int64),
                ("ws1_elems", C.c_int64), ("ws2_elems", C.c_int64), ("out_elems", C.c_int64),
                ("t4", C.c_void_p), ("c4", C.c_void_p), ("items4", C.c_void_p),
                ("n_items4", C.c_int64)]


class TcPlan(C.Structure):
    _fields_ = [("cvt", C.c_void_p), ("cvt_items", C.c_void_p), ("n_cvt_items", C.c_int64),
                ("t1", C.c_void_p), ("s1", C.c_void_p), ("tiles1", C.c_void_p),
                ("n_tiles1", C.c_int64),
                ("t2", C.c_void_p), ("c2", C.c_void_p), ("items2", C.c_void_p),
                ("n_items2", C.c_int64),
                ("t3", C.c_void_p), ("s3", C.c_void_p), ("tiles3", C.c_void_p),
                ("n_tiles3", C.c_int64),
                ("maps", C.c_void_p), ("stage", C.c_void_p), ("lo_off", C.c_int64),
                ("y32", C.c_void_p), ("err", C.c_void_p), ("passes", C.c_int32),
                ("bn3", C.c_int32)]


_P, _I64, _I32, _D = C.c_void_p, C.c_int64, C.c_int32, C.c_double
_SIGS = {
    "tnk_version": ([], C.c_char_p),
    "tnk_last_error": ([], C.c_char_p),
    "tnk_struct_sizes": ([_P], C.c_int),
    "tnk_contract3_f64": ([_P, _P, _P, _P, _P, _P, _I64, _P], C.c_int),
    "tnk_apply_two_site_f64": ([_P, _P, _P, _P, _P, _P, _I64, _P], C.c_int),
    "tnk_apply_one_site_f64": ([_P, _P, _P, _P, _P, _P, _I64, _P], C.c_int),
    "tnk_update_left_env_f64": ([_P, _P, _P, _P, _P, _I64, _P], C.c_int),
    "tnk_update_right_env_f64": ([_P, _P, _P, _P, _P, _I64, _P], C.c_int),
    "tnk_grouped_gemm_f64": ([_P, _P, _P, _I64, _P, _P, _P, _P, _P, _P], C.c_int),
    "tnk_combine_f64": ([_P, _P, _P, _I64, _P, _P, _P], C.c_int),
    "tnk_dot_f64": ([_P, _P, _I64, _P, _P, _P], C.c_int),
    "tnk_nrm2_f64": ([_P, _I64, _P, _P, _P], C.c_int),
    "tnk_multidot_f64": ([_P, _I64, _I32, _P, _I64, _P, _P, _P], C.c_int),
    "tnk_gemv_sub_f64": ([_P, _I64, _I32, _P, _P, _I64, _P], C.c_int),
    "tnk_axpby_f64": ([_P, _P, _I64, _P, _D, _P, _D, _P], C.c_int),
    "tnk_scale_div_f64": ([_P, _P, _I64, _P, _D, _P], C.c_int),
    "tnk_cgs_pass_f64": ([_P, _I64, _I32, _P, _P, _I64, _P, _I32, _P, _P, _P], C.c_int),
    "tnk_cgs_pass_f32": ([_P, _I64, _I32, _P, _P, _I64, _P, _I32, _P, _P, _P], C.c_int),
    "tnk_scale_div_seg_f64": ([_P, _P, _P, _P, _I32, _I64, _P, _I64, _D, _P], C.c_int),
    "tnk_cgs_pass_seg_f64": ([_P, _I64, _I32, _P, _P, _P, _P, _I32, _I64, _I64, _P, _I32, _P,
                              _P, _P], C.c_int),
    "tnk_scale_div_f32": ([_P, _P, _I64, _P, _D, _P], C.c_int),
    "tnk_rotate_f32": ([_P, _I64, _I32, _P, _I32, _P, _I64, _I64, _P], C.c_int),
    "tnk_svd_gram_ws_f64": ([_I64, _I64, _P], C.c_int),
    "tnk_svd_gram_f64": ([_P, _I64, _I64, _P, _P, _P, _P, _I64, _P, _P], C.c_int),
    "tnk_svd_gram_ws2_f64": ([_I64, _I64, _I32, _P], C.c_int),
    "tnk_svd_gram2_f64": ([_P, _I64, _I64, _I32, _P, _P, _P, _P, _I64, _P, _P], C.c_int),
    "tnk_svd_gram_ws_f32": ([_I64, _I64, _P], C.c_int),
    "tnk_svd_gram_f32": ([_P, _I64, _I64, _P, _P, _P, _P, _I64, _P, _P], C.c_int),
    "tnk_apply_two_site_f64_noalloc": ([_P, _P, _P, _P, _P, _P], C.c_int),
    "tnk_noalloc_scratch_elems": ([_P], C.c_int),
    "tnk_apply_two_site_tc": ([_P, _P, _P, _P], C.c_int),
    "tnk_stage_f32": ([_P, _P, _I64, _P, _P, _I64, _I32, _P], C.c_int),
    "tnk_tc_encode_tmaps": ([_P, _P, _I64, _P], C.c_int),
    "tnk_tc_encode_tmaps_box": ([_P, _P, _I64, _P], C.c_int),
    "tnk_grouped_gemm_tc": ([_P, _P, _P, _I64, _P, _P, _P, _I32, _P], C.c_int),
    "tnk_tc_schedule": ([_I32], C.c_int),
    "tnk_grouped_gemm_tc_bn": ([_P, _P, _P, _I64, _P, _P, _P, _I32, _I32, _P], C.c_int),
    "tnk_combine_f32": ([_P, _P, _P, _I64, _P, _P, _I64, _I32, _P], C.c_int),
    "tnk_ff_split": ([_P, _P, _I64, _P], C.c_int),
    "tnk_contract3_ff": ([_P, _P, _P, _P, _P, _P, _I64, _P], C.c_int),
    "tnk_apply_two_site_ff": ([_P, _P, _P, _P, _P, _P, _I64, _P], C.c_int),
    "tnk_grouped_gemm_ff": ([_P, _P, _P, _I64, _P, _P, _P, _P, _P, _P], C.c_int),
    "tnk_zdot_f64": ([_P, _P, _I64, _P, _P, _P], C.c_int),
    "tnk_zmultidot_f64": ([_P, _I64, _I32, _P, _I64, _P, _P, _P], C.c_int),
    "tnk_zgemv_sub_f64": ([_P, _I64, _I32, _P, _P, _I64, _P], C.c_int),
    "tnk_zaxpby_f64": ([_P, _P, _I64, _P, _D, _P, _D, _P], C.c_int),
    "tnk_gemm_f64_variant": ([_I32], C.c_int),
    "tnk_tridiag_eig_f64": ([_P, _P, _I64, _I64, _I64, _I64, _P, _P, _P, _P], C.c_int),
    "tnk_sytrd_limits": ([_I32, _P], C.c_int),
    "tnk_sytrd_batched_f64": ([_P, _I32, _I32, _I32, _P, _P, _P, _P, _P], C.c_int),
    "tnk_ormtr_batched_f64": ([_P, _P, _I32, _I32, _P, _P, _P, _P], C.c_int),
    "tnk_gebrd_limits": ([_I32, _P], C.c_int),
    "tnk_gebrd_batched_f64": ([_P, _I32, _I32, _I32, _I32, _P, _P, _P, _P, _P], C.c_int),
    "tnk_ormqr_batched_f64": ([_P, _P, _I32, _I32, _P, _P, _P, _P], C.c_int),
    "tnk_apply_plan_build": ([_P, _P], C.c_int),
    "tnk_plan_tc_build": ([_P, _I64, _P, _P, _I64, _P, _I64, _P, _P], C.c_int),
    "tnk_env_plan_build": ([_P, _P], C.c_int),
    "tnk_tensordot_plan_build": ([_P, _P, _P, _I32, _P], C.c_int),
    "tnk_plan_split_k": ([_P, _I64, _P, _I64, _I32, _I32, _I32, _I32, _P], C.c_int),
    "tnk_planb_table": ([_P, _I32, _P, _P], C.c_int),
    "tnk_planb_scalars": ([_P, _P], C.c_int),
    "tnk_planb_free": ([_P], None),
}

_lib = None
_load_error = None


def exported_symbols():
    """Names the header declares (every one must be exported by the library)."""
    return sorted(_SIGS)


def load(path: str = LIB_PATH):
    """Load and type the library (once). Raises LibraryMissing if it cannot be loaded."""
    global _lib, _load_error
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        _load_error = f"{path} not found; build it with `python -m tnkit_gb300.build`"
        raise LibraryMissing(_load_error)
    lib = C.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    sizes = (C.c_int64 * 6)()
    lib.tnk_struct_sizes(C.cast(sizes, C.c_void_p))
    mine = [d.itemsize for d in (GEMM_TASK, GEMM_SEG, GEMM_TILE, COMB_TASK, COMB_TERM,
                                 COMB_ITEM)]
    if list(sizes) != mine:
        raise LibraryMissing(f"table layout mismatch: library {list(sizes)} vs host {mine}")
    _lib = lib
    return lib


def lib():
    return _lib if _lib is not None else load()


def check(rc: int, where: str):
    if rc != TNK_OK:
        raise TnkError(rc, where, lib().tnk_last_error().decode(errors="replace"))


def ptr(t) -> int:
    """Device (or host) address of a torch tensor, or 0 for None."""
    return 0 if t is None else int(t.data_ptr())


def stream_ptr(stream=None) -> int:
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return int(s.cuda_stream)
