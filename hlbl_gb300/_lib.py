"""ctypes binding of libhlbl_gb300.so (the C ABI of include/hlbl_gb300.h).

The library is the product: there is no fallback. If it is missing this
module raises at import, naming the build command. HLBL_GB300_LIB selects
another build of it (for example one linked with a KQED).
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB as _DEFAULT_LIB

LIB = os.environ.get("HLBL_GB300_LIB") or _DEFAULT_LIB

I4 = C.c_int * 4


class TrainConfig(C.Structure):
    """hlbl_train_config (include/hlbl_gb300.h)."""
    _fields_ = [("n_samples", C.c_longlong), ("batch", C.c_int), ("steps", C.c_int),
                ("lr", C.c_float), ("seed", C.c_uint64), ("radius", C.c_float),
                ("n_valid", C.c_longlong), ("bound", C.c_double)]


class TrainReport(C.Structure):
    """hlbl_train_report (include/hlbl_gb300.h)."""
    _fields_ = [("final_loss", C.c_float), ("max_rel_err_net", C.c_double),
                ("rms_rel_err_net", C.c_double), ("max_rel_err_base", C.c_double),
                ("rms_rel_err_base", C.c_double), ("r0", C.c_double),
                ("train_seconds", C.c_double), ("r1", C.c_double)]


class HlblError(RuntimeError):
    """A C-ABI call returned a nonzero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"hlbl error {code}: {msg}")
        self.code = code


def _load() -> C.CDLL:
    if not os.path.exists(LIB):
        raise ImportError(f"{LIB} is missing: build it with `python -m hlbl_gb300.build`")
    lib = C.CDLL(LIB)
    vp, i4p, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
    sigs = {
        "hlbl_last_error": (C.c_char_p, []),
        "hlbl_version": (C.c_char_p, []),
        "hlbl_ctx_create": (C.c_int, [C.POINTER(vp), i4p, i4p, i4p, C.c_double, C.c_int]),
        "hlbl_ctx_destroy": (None, [vp]),
        "hlbl_ctx_set_stream": (C.c_int, [vp, vp]),
        "hlbl_ctx_check": (C.c_int, [vp]),
        "hlbl_selftest_wait_timeout": (C.c_int, [vp]),
        "hlbl_kernel_sum": (C.c_int, [vp, vp, vp, i4p, i4p, C.c_double, C.c_int, dp]),
        "hlbl_kernel_sum_async": (C.c_int, [vp, vp, vp, i4p, i4p, C.c_double, C.c_int, vp]),
        "hlbl_cu_dzu_dzsu": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, i4p, i4p, i4p, i4p]),
        "hlbl_cu_dzu_dzsu_noalloc": (C.c_int, [vp, vp, vp, vp, C.c_int, i4p, i4p, i4p, i4p, vp]),
        "hlbl_cu_4pt_contraction": (C.c_int, [vp, vp, vp, vp, vp, vp, C.c_int, i4p, i4p,
                                              C.c_double, i4p, i4p, i4p]),
        "hlbl_insert_gammas": (C.c_int, [vp, vp, vp, vp, vp]),
        "hlbl_reserve_kernel_memory": (C.c_int, [vp, C.POINTER(C.c_size_t)]),
        "hlbl_fill_random_block": (C.c_int, [vp, vp, C.c_uint64]),
        "hlbl_fill_gaussian_block": (C.c_int, [vp, vp, C.c_uint64]),
        "hlbl_source_seed": (C.c_uint64, [C.c_uint64, i4p]),
        "hlbl_block_length": (C.c_size_t, [vp]),
        "hlbl_ctx_set_profiling": (C.c_int, [vp, C.c_int]),
        "hlbl_kernel_sums_batched": (C.c_int, [vp, vp, C.c_int, C.POINTER(vp), i4p, i4p,
                                               C.c_double, C.c_int, vp]),
        "hlbl_ctx_set_batch_group": (C.c_int, [vp, C.c_int]),
        "hlbl_ctx_set_tensor_cores": (C.c_int, [vp, C.c_int]),
        "hlbl_ctx_set_tc_fp16": (C.c_int, [vp, C.c_int]),
        "hlbl_f32_tile_copy": (C.c_int, [vp, vp, vp]),
        "hlbl_f32_block_length": (C.c_size_t, [vp]),
        "hlbl_kernel_sums_batched_f32": (C.c_int, [vp, vp, C.c_int, C.POINTER(vp), i4p, i4p, C.c_double, vp]),
        "hlbl_autotune_f32": (C.c_int, [vp, vp, C.c_int, C.POINTER(vp), i4p, i4p, C.c_double, vp,
                                        C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]),
        "hlbl_ctx_set_qed_fp32": (C.c_int, [vp, C.c_int, C.c_double]),
        "hlbl_ctx_set_p1f32_variant": (C.c_int, [vp, C.c_int, C.c_int]),
        "hlbl_ctx_reserve": (C.c_int, [vp, C.c_int]),
        "hlbl_stage_async": (C.c_int, [vp, vp, vp, C.c_size_t, C.c_int]),
        "hlbl_autotune": (C.c_int, [vp, vp, C.c_int, C.POINTER(vp), i4p, i4p, C.c_double, vp,
                                    C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), dp]),
        "hlbl_graph_begin": (C.c_int, [vp]),
        "hlbl_graph_end": (C.c_int, [vp, C.POINTER(vp)]),
        "hlbl_graph_launch": (C.c_int, [vp, vp]),
        "hlbl_graph_destroy": (None, [vp]),
        "hlbl_surrogate_create": (C.c_int, [C.POINTER(vp), C.c_int, C.c_double, C.c_uint64]),
        "hlbl_surrogate_destroy": (None, [vp]),
        "hlbl_surrogate_train": (C.c_int, [vp, C.POINTER(TrainConfig), C.POINTER(TrainReport)]),
        "hlbl_surrogate_params": (C.c_int, [vp, vp, vp, C.c_int]),
        "hlbl_surrogate_gradients": (C.c_int, [vp, vp, vp, C.c_int, vp, C.POINTER(C.c_float)]),
        "hlbl_surrogate_eval": (C.c_int, [vp, vp, C.c_int, vp]),
        "hlbl_ctx_set_qed": (C.c_int, [vp, C.c_int, vp, C.c_double]),
        "hlbl_ctx_set_qed_kernel": (C.c_int, [vp, C.c_int, C.c_uint64]),
        "hlbl_ctx_qed_fallbacks": (C.c_int, [vp, C.POINTER(C.c_ulonglong)]),
        "hlbl_ctx_kernel_times": (C.c_int, [vp, dp, C.POINTER(C.c_longlong)]),
        "hlbl_measure_fma_peak": (C.c_int, [C.c_int, C.c_int, dp]),
        "hlbl_2p2_lmax": (C.c_int, [vp]),
        "hlbl_2p2_reserve": (C.c_int, [vp]),
        "hlbl_ctx_set_2p2_r64": (C.c_int, [vp, C.c_double]),
        "hlbl_pieces_2p2": (C.c_int, [vp, vp, i4p, vp, C.c_int, C.c_double, C.c_int, vp, vp]),
        "hlbl_pieces_2p2_async": (C.c_int, [vp, vp, i4p, vp, C.c_int, C.c_double, C.c_int, vp, vp]),
        "hlbl_pieces_2p2_f32": (C.c_int, [vp, vp, i4p, vp, C.c_int, C.c_double, vp, vp]),
        "hlbl_compute_2p2": (C.c_int, [vp, vp, vp, vp, C.c_int, i4p, vp, C.c_int, C.c_double, C.c_int]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def check(rc: int) -> None:
    if rc != 0:
        raise HlblError(rc, lib.hlbl_last_error().decode())


def i4(v) -> "C.Array":
    v = [int(a) for a in v]
    if len(v) != 4:
        raise ValueError("expected 4 coordinates (t, x, y, z)")
    return I4(*v)


def ptr(x) -> int:
    """Device address of a torch tensor (or an int address)."""
    if isinstance(x, int):
        return x
    return int(x.data_ptr())
