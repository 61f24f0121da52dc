"""ctypes binding of libmpsxx_gb300.so (the C ABI in include/mpsxx_gb300.h).

The shared library is built in-tree by ``mpsxx_gb300.build``; loading fails
loudly when it is missing — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libmpsxx_gb300.so"

c_int_p = C.POINTER(C.c_int)
c_i64_p = C.POINTER(C.c_int64)
c_dbl_p = C.POINTER(C.c_double)
vp = C.c_void_p
vpp = C.POINTER(C.c_void_p)

# name: (restype, argtypes)
SIGNATURES = {
    "mpsxx_version": (C.c_int, []),
    "mpsxx_last_error": (C.c_char_p, []),
    "mpsxx_context_create": (C.c_int, [C.c_int, vp, vpp]),
    "mpsxx_context_destroy": (C.c_int, [vp]),
    "mpsxx_context_sync": (C.c_int, [vp]),
    "mpsxx_context_counters": (C.c_int, [vp, c_i64_p, c_dbl_p, c_i64_p]),
    "mpsxx_context_set_truncation": (C.c_int, [vp, C.c_double]),
    "mpsxx_context_set_split_refinement": (C.c_int, [vp, C.c_double, C.c_int]),
    "mpsxx_context_tuning": (C.c_int, [vp, c_dbl_p, C.c_int, C.POINTER(C.c_int)]),
    "mpsxx_context_set_sigma_schedule": (C.c_int, [vp, C.c_int64, C.c_int, C.c_int]),
    "mpsxx_context_set_sigma_operator_format": (C.c_int, [vp, C.c_int]),
    "mpsxx_context_set_svd_routes": (C.c_int, [vp, C.c_int, C.c_int]),
    "mpsxx_context_set_plan_cache": (C.c_int, [vp, C.c_int64]),
    "mpsxx_context_set_device_timeout": (C.c_int, [vp, C.c_int64]),
    "mpsxx_sigma_plan_stats": (C.c_int, [vp, vp, vp, vp, c_dbl_p, C.c_int, C.POINTER(C.c_int)]),
    "mpsxx_mpo_gradient": (C.c_int, [vp, vp, vp, vp, vp, vp, c_dbl_p, c_dbl_p]),
    "mpsxx_merge_rows": (C.c_int, [vp, vp, vpp]),
    "mpsxx_diagonalize_projected": (C.c_int, [vp, vp, vp, vp, vp, C.c_double, C.c_int, vpp, vpp, c_dbl_p, c_dbl_p,
                                              C.POINTER(C.c_int)]),
    "mpsxx_tensor_accumulate": (C.c_int, [vp, C.c_double, vp, vp]),
    "mpsxx_optimize_twosite_merged_batch": (C.c_int, [vp, C.c_int, C.POINTER(C.c_int), vpp, vpp, vpp, vpp, vpp, vpp,
                                                      C.c_double, C.POINTER(C.c_int), c_dbl_p, c_dbl_p, vpp, vpp,
                                                      vpp, c_dbl_p]),
    "mpsxx_expand_rows": (C.c_int, [vp, vp, vp, vpp]),
    "mpsxx_context_profile": (C.c_int, [vp, C.c_int, C.c_int, c_dbl_p, C.c_int, C.POINTER(C.c_int)]),
    "mpsxx_context_set_precision": (C.c_int, [vp, C.c_int]),
    "mpsxx_context_get_precision": (C.c_int, [vp, c_int_p]),
    "mpsxx_tensor_create": (C.c_int, [vp, C.c_int, c_int_p, c_int_p, c_int_p, c_int_p, C.c_int64, c_i64_p, vpp]),
    "mpsxx_tensor_create_like": (C.c_int, [vp, vp, vpp]),
    "mpsxx_tensor_destroy": (C.c_int, [vp]),
    "mpsxx_tensor_info": (C.c_int, [vp, c_int_p, c_int_p, c_i64_p, c_i64_p]),
    "mpsxx_tensor_shape": (C.c_int, [vp, c_int_p, c_int_p, c_int_p]),
    "mpsxx_tensor_blocks": (C.c_int, [vp, c_i64_p, c_i64_p]),
    "mpsxx_tensor_upload": (C.c_int, [vp, c_dbl_p]),
    "mpsxx_tensor_download": (C.c_int, [vp, c_dbl_p]),
    "mpsxx_tensor_device_ptr": (C.c_int, [vp, C.POINTER(c_dbl_p)]),
    "mpsxx_gemm_tasks": (C.c_int, [C.c_int, C.c_int, vp, vp, C.c_int, c_i64_p, c_i64_p, c_i64_p, c_i64_p, c_i64_p,
                                   c_i64_p]),
    "mpsxx_compute_sigma_vector": (C.c_int, [vp, vp, vp, vp, vp]),
    "mpsxx_compute_diagonal_elements": (C.c_int, [vp, vp, vp, vp]),
    "mpsxx_renormalize": (C.c_int, [vp, C.c_int, vp, vp, vp, vpp]),
    "mpsxx_compute_merged_operator": (C.c_int, [vp, C.c_int, vp, vp, vpp]),
    "mpsxx_diagonalize": (C.c_int, [vp, vp, vp, vp, vp, C.c_double, c_dbl_p, c_int_p]),
    "mpsxx_canonicalize": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_double, vpp, vpp]),
    "mpsxx_optimize_twosite_merged": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp, vp, C.c_double, C.c_int,
                                                C.c_double, c_dbl_p, vpp, vpp, vpp, c_dbl_p]),
    "mpsxx_make_noise": (C.c_int, [vp, vp, C.c_double]),
    "mpsxx_compute_sigma_vector_onesite": (C.c_int, [vp, vp, vp, vp, vp, vpp]),
    "mpsxx_compute_sigma_vector_twosite": (C.c_int, [vp, vp, vp, vp, vp, vp, vpp]),
    "mpsxx_compute_sigma_vector_overlap": (C.c_int, [vp, vp, vp, vp, vpp]),
    "mpsxx_renormalize_mpo": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vpp]),
    "mpsxx_renormalize_overlap": (C.c_int, [vp, C.c_int, vp, vp, vp, vpp]),
    "mpsxx_compute_guesswave": (C.c_int, [vp, C.c_int, vp, vp, vp, vpp]),
    "mpsxx_compute_diagonal_elements_onesite": (C.c_int, [vp, vp, vp, vp, vp]),
    "mpsxx_compute_diagonal_elements_twosite": (C.c_int, [vp, vp, vp, vp, vp, vp]),
    "mpsxx_noise_sequence": (C.c_int, [C.c_int64, c_dbl_p]),
    "mpsxx_merge_cols": (C.c_int, [vp, vp, vpp]),
    "mpsxx_gemm": (C.c_int, [vp, C.c_int, C.c_int, C.c_double, vp, vp, C.c_int, vpp]),
    "mpsxx_expand_cols": (C.c_int, [vp, vp, vp, vpp]),
    "mpsxx_normalize": (C.c_int, [vp, vp, c_dbl_p]),
    "mpsxx_sigma_device_time": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, c_dbl_p]),
    "mpsxx_multidot_noalloc": (C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int64, C.c_int64, vp, vp]),
    "mpsxx_merge_wavefunction":(C.c_int, [vp, vp, vp, vp, vp, vp, vp, vpp]),
    "mpsxx_expand_wavefunction": (C.c_int, [vp, vp, vp, vp, vp, vp, vp, vpp, vpp]),
}

STATUS = {0: "OK", 1: "QSHAPE_MISMATCH", 2: "ALLOC", 3: "NO_CONVERGENCE", 4: "DEVICE_TIMEOUT",
          5: "INVALID_ARGUMENT", 6: "CUDA", 7: "SOLVER", 8: "INTERNAL"}


class MpsxxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built: run mpsxx_gb300.build.build() (nvcc, sm_103a)")
        h = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        _LIB = h
    return _LIB


def check(code: int):
    if code != 0:
        msg = lib().mpsxx_last_error()
        raise MpsxxError(code, msg.decode() if msg else "")
