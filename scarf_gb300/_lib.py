"""ctypes binding of ``libscarfgpu.so`` (the C ABI declared in include/scarf_gb300.h).

The library is loaded from the package's ``_build`` directory. There is no
fallback: when it is missing or fails to load, every GPU entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "_build" / "libscarfgpu.so"

SG_OK = 0
SG_ERR_ARG = -1
SG_ERR_OOM = -2
SG_ERR_CUDA = -3
SG_ERR_TIMEOUT = -4
SG_ERR_BUDGET = -5
SG_ERR_UNSUPPORTED = -6

SG_F32, SG_BF16, SG_F64 = 0, 1, 2
SG_PLAIN, SG_PRECISION = 0, 1
SG_NORM_LOG1P = 1
SG_NORM_RENORM_SUBSET = 2
SG_UNION_UPPER_ONLY = 1

vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
u32 = C.c_uint32
u64 = C.c_uint64
f32 = C.c_float
f64 = C.c_double
sz = C.c_size_t

# name -> (restype, argtypes)
SIGNATURES = {
    "sg_version": (C.c_int, []),
    "sg_last_error": (C.c_char_p, []),
    "sg_create": (C.c_int, [C.c_int, sz, C.POINTER(vp)]),
    "sg_destroy": (C.c_int, [vp]),
    "sg_workspace_bytes": (sz, [vp]),
    "sg_kernel_launches": (C.c_ulonglong, []),
    "sg_profile": (C.c_int, [vp, C.c_int]),
    "sg_profile_reset": (C.c_int, [vp]),
    "sg_profile_query": (C.c_int, [vp, C.c_char_p, C.POINTER(f64), C.POINTER(C.c_longlong)]),
    "sg_normalize_csr": (C.c_int, [vp, vp, vp, vp, i64, vp, i64, i32, vp, f32, vp, f64, u32, vp, i64, i32, vp,
                                   vp, vp, vp]),
    "sg_zstats": (C.c_int, [vp, vp, vp, i64, i32, vp, vp, vp, vp, vp]),
    "sg_covariance": (C.c_int, [vp, vp, i64, i32, i64, vp, vp, vp, i32, vp, vp, vp]),
    "sg_pca_basis": (C.c_int, [vp, vp, vp, i64, i32, i32, vp, vp, vp, i32, vp, i32, vp]),
    "sg_pca_basis_mixed": (C.c_int, [vp, vp, vp, i64, i32, i32, vp, vp, vp, i32, vp, i32, vp]),
    "sg_pca_basis_filter": (C.c_int, [vp, vp, vp, i64, i32, i32, vp, vp, vp, i32, vp, i32, vp]),
    "sg_pca_filter_residual": (C.c_double, [vp]),
    "sg_set_autotune": (C.c_int, [vp, C.c_int]),
    "sg_knn_last_splits": (C.c_int, [vp]),
    "sg_knn_last_locality": (C.c_int, [vp]),
    "sg_set_wait_limit": (C.c_int, [vp, u32]),
    "sg_test_idle_mma": (C.c_int, [vp]),
    "sg_project": (C.c_int, [vp, vp, i64, i32, i64, vp, vp, vp, i32, i32, vp, i32, vp, i32, i32, vp]),
    "sg_knn": (C.c_int, [vp, vp, i64, vp, i64, i32, i32, i32, i64, i32, i32, vp, vp, vp, vp]),
    "sg_smooth": (C.c_int, [vp, vp, vp, i64, i32, f64, f64, i64, vp, vp, vp]),
    "sg_smooth_noalloc": (C.c_int, [vp, vp, i64, i32, f64, f64, i64, vp, vp, vp]),
    "sg_fuzzy_union": (C.c_int, [vp, vp, vp, i64, i64, i32, i32, f64, u32, vp, vp, vp, i64, vp]),
    "sg_serve_create": (C.c_int, [C.c_int, vp, vp, vp, i32, i32, i32, vp, i64, i32, vp, i64, vp, i32, i32, f64, u32,
                                  i32, sz, i32, C.POINTER(vp)]),
    "sg_serve_submit": (C.c_int, [vp, vp, vp, vp, i64, C.POINTER(i64)]),
    "sg_serve_poll": (C.c_int, [vp, i64, C.POINTER(i32)]),
    "sg_serve_wait": (C.c_int, [vp, i64, i64]),
    "sg_serve_result": (C.c_int, [vp, i64, vp, vp]),
    "sg_serve_stats": (C.c_int, [vp, C.POINTER(i64), C.POINTER(i64)]),
    "sg_serve_destroy": (C.c_int, [vp]),
    "sg_blosc_decode": (C.c_int, [vp, vp, vp, i32, vp, i64, vp, vp]),
    "sg_chunks_to_csr": (C.c_int, [vp, vp, i64, i32, i32, i64, i64, vp, vp, vp, i64, C.POINTER(i64), vp]),
    "sg_blosc_encode": (C.c_int, [vp, vp, vp, i32, i32, i32, i32, vp, i64, vp, vp]),
    "sg_blosc_encode_bound": (C.c_int64, [vp, i32, i32]),
    "sg_kmeans_minibatch": (C.c_int, [vp, vp, i64, i32, i32, i32, i32, u64, vp, vp, vp]),
    "sg_calc_snn": (C.c_int, [vp, vp, i64, i32, vp, vp]),
    "sg_merge_graphs": (C.c_int, [vp, i32, vp, vp, vp, i64, i32, vp, vp, vp]),
    "sg_umap_layout": (C.c_int, [vp, vp, vp, vp, i64, i64, i32, vp, i32, f32, f32, f32, f32, f32, u64, i32, vp]),
}

_lock = threading.Lock()
_lib = None


class LibraryMissing(RuntimeError):
    pass


def load():
    """Load the CUDA library once; raise when it is absent (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = os.environ.get("SCARF_GB300_LIB", str(LIB_PATH))
        if not os.path.exists(path):
            raise LibraryMissing(
                f"scarf_gb300 CUDA library not found at {path}; build it with "
                "`python -m scarf_gb300.build` (there is no CPU fallback)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def exported_symbols():
    return list(SIGNATURES)


class GpuError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


def check(status: int):
    if status == SG_OK:
        return
    msg = load().sg_last_error().decode(errors="replace")
    if status == SG_ERR_ARG:
        raise ValueError(msg)
    if status in (SG_ERR_OOM, SG_ERR_BUDGET):
        raise MemoryError(msg)
    if status == SG_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise GpuError(status, msg)
