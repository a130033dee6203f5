"""ctypes declarations of include/accspmm.h (libaccspmm.so).

Loading fails loudly when the library has not been built: there is no Python
or CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
# ACCSPMM_LIB selects another build of the library (same ABI)
LIB_PATH = os.environ.get("ACCSPMM_LIB") or os.path.join(PKG, "libaccspmm.so")
# the measurement build: the same ABI plus the variant kernels and the gather floor
LAB_PATH = os.path.join(PKG, "libaccspmm_lab.so")
HEADER = os.path.join(ROOT, "include", "accspmm.h")

u32 = C.c_uint32
i32 = C.c_int32
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)
vp = C.c_void_p

SUCCESS = 0
ERROR_OPEN_FILE = 2
ERROR_READ_MTX = 3
ERROR_ARGS = 4
MM_LOADING_FILE_ERROR = -1
MM_READ_BANNER_ERROR = -2
ERROR_INVALID_VALUE = 30
ERROR_ALLOC = 31
ERROR_CUDA = 32
ERROR_UNSUPPORTED = 33
ERROR_OVERFLOW = 34
ERROR_TIMEOUT = 35
ERROR_ADMISSION = 36
ERROR_CANCELLED = 37
ERROR_FORMAT = 38
PREC_TF32 = 0
PREC_3XTF32 = 1
OPT_PACK = 0
OPT_PREFETCH = 1
OPT_SCHEDULE = 2
OPT_SLICE_WIDTH = 3
OPT_CTAS_PER_SM = 4
OPT_TILE_RING = 5
OPT_WINDOWS_PER_CTA = 6
OPT_HOST_SLICE_WIDTH = 7
OPT_HOST_DIRECT_C = 8
OPT_KERNEL = 9
KERNELS = {"direct": 0, "pipe": 1, "bulk": 2, "lean": 3, "db": 4, "tma": 5, "staged": 6}
ACT_NONE = 0
ACT_RELU = 1
HOST = 0
DEVICE = 1


class COO(C.Structure):
    _fields_ = [("rows", u32), ("cols", u32), ("nnz", u32), ("row", u32p), ("col", u32p),
                ("data", f32p), ("space", i32), ("owned", i32)]


class CSR(C.Structure):
    _fields_ = [("rows", u32), ("cols", u32), ("nnz", u32), ("row_ptr", u32p),
                ("col_idx", u32p), ("data", f32p), ("space", i32), ("owned", i32)]


class METCF(C.Structure):
    _fields_ = [("rows", u32), ("cols", u32), ("nnz", u32), ("num_windows", u32),
                ("num_tiles", u32), ("row_window_offset", u32p), ("tc_offset", u32p),
                ("tc_local_bit", u64p), ("sparse_a2b", u32p), ("data", f32p),
                ("space", i32), ("owned", i32)]


class ADPBME(C.Structure):
    _fields_ = [("rows", u32), ("cols", u32), ("nnz", u32), ("num_tiles", u32),
                ("num_groups", u32), ("group_offset", u32p), ("tc_offset", u32p),
                ("row_indices", u32p), ("tc_local_bit", u64p), ("sparse_a2b", u32p),
                ("data", f32p), ("space", i32), ("owned", i32)]


class TUNE(C.Structure):
    _fields_ = [("kernel", i32), ("slice_width", u32), ("windows_per_cta", u32),
                ("best_ms", C.c_float), ("default_ms", C.c_float), ("candidates", u32),
                ("ctas_per_sm", u32), ("tile_ring", i32), ("packed_b", i32)]


class SERVERCFG(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_batch", u32), ("streams", u32)]


class SERVERSTATS(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("cancelled", C.c_uint64), ("launches", C.c_uint64), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("mean_ms", C.c_double), ("max_ms", C.c_double),
                ("throughput_rps", C.c_double), ("mean_batch", C.c_double),
                ("peak_bytes", C.c_size_t)]


class BATCHITEM(C.Structure):
    _fields_ = [("metcf", C.POINTER(METCF)), ("B", vp), ("C", vp), ("K", u32)]


_SIGS = {
    "accspmm_version": ([], C.c_char_p),
    "accspmm_last_error": ([], C.c_char_p),
    "accspmm_read_mtx": ([C.c_char_p, C.POINTER(COO)], C.c_int),
    "accspmm_csr_from_coo": ([C.POINTER(COO), C.POINTER(CSR), vp], C.c_int),
    "accspmm_metcf_from_csr": ([C.POINTER(CSR), C.POINTER(METCF), vp], C.c_int),
    "accspmm_adpbme_from_metcf": ([C.POINTER(METCF), u32, u32, u32, u32, C.POINTER(ADPBME), vp],
                                  C.c_int),
    "accspmm_balance_strategy": ([C.POINTER(METCF), C.POINTER(C.c_int), vp], C.c_int),
    "accspmm_adaptive_c_rows": ([C.POINTER(ADPBME), u32p, vp], C.c_int),
    "accspmm_metcf_copy": ([C.POINTER(METCF), i32, C.POINTER(METCF), vp], C.c_int),
    "accspmm_csr_copy": ([C.POINTER(CSR), i32, C.POINTER(CSR), vp], C.c_int),
    "accspmm_coo_copy": ([C.POINTER(COO), i32, C.POINTER(COO), vp], C.c_int),
    "accspmm_adpbme_copy": ([C.POINTER(ADPBME), i32, C.POINTER(ADPBME), vp], C.c_int),
    "accspmm_reorder_rcm": ([C.POINTER(CSR), u32p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], C.c_int),
    "accspmm_csr_permute": ([C.POINTER(CSR), u32p, C.POINTER(CSR)], C.c_int),
    "accspmm_dense_permute_rows": ([vp, vp, vp, u32, u32, i32, vp], C.c_int),
    "accspmm_metcf_save": ([C.POINTER(METCF), C.c_char_p, vp], C.c_int),
    "accspmm_metcf_load": ([C.c_char_p, i32, C.POINTER(METCF), vp], C.c_int),
    "accspmm_adpbme_save": ([C.POINTER(ADPBME), C.c_char_p, vp], C.c_int),
    "accspmm_adpbme_load": ([C.c_char_p, i32, C.POINTER(ADPBME), vp], C.c_int),
    "accspmm_coo_destroy": ([C.POINTER(COO)], None),
    "accspmm_csr_destroy": ([C.POINTER(CSR)], None),
    "accspmm_metcf_destroy": ([C.POINTER(METCF)], None),
    "accspmm_adpbme_destroy": ([C.POINTER(ADPBME)], None),
    "accspmm_spmm_tf32": ([C.POINTER(METCF), vp, vp, u32, i32, vp], C.c_int),
    "accspmm_spmm_adaptive": ([C.POINTER(ADPBME), vp, vp, u32, u32, i32, vp], C.c_int),
    "accspmm_device_status": ([vp], C.c_int),
    "accspmm_selftest_bounded_wait": ([C.c_uint32, vp], C.c_int),
    "accspmm_autotune_metcf": ([C.POINTER(METCF), vp, vp, u32, i32, vp, C.POINTER(TUNE)], C.c_int),
    "accspmm_autotune_clear": ([], None),
    "accspmm_server_create": ([C.POINTER(METCF), u32, C.POINTER(SERVERCFG), C.POINTER(vp)], C.c_int),
    "accspmm_server_submit": ([vp, u32, vp, vp, u32, i32, u32, C.POINTER(C.c_uint64)], C.c_int),
    "accspmm_server_wait": ([vp, C.c_uint64, i32], C.c_int),
    "accspmm_server_cancel": ([vp, C.c_uint64], C.c_int),
    "accspmm_server_stats": ([vp, C.POINTER(SERVERSTATS)], C.c_int),
    "accspmm_server_reset_stats": ([vp], C.c_int),
    "accspmm_server_destroy": ([vp], None),
    "accspmm_batch_create": ([C.POINTER(BATCHITEM), u32, i32, C.POINTER(vp)], C.c_int),
    "accspmm_batch_run": ([vp, vp], C.c_int),
    "accspmm_batch_capture": ([vp, vp], C.c_int),
    "accspmm_batch_launch_graph": ([vp, vp], C.c_int),
    "accspmm_batch_info": ([vp, u32p, u32p, u32p], C.c_int),
    "accspmm_batch_destroy": ([vp], None),
    "accspmm_spmm_bias_act": ([C.POINTER(METCF), vp, vp, u32, i32, vp, i32, vp], C.c_int),
    "accspmm_gcn_layer": ([C.POINTER(METCF), vp, u32, vp, u32, vp, i32, vp, i32, vp], C.c_int),
    "accspmm_dense_matmul": ([vp, u32, u32, vp, u32, vp, i32, vp], C.c_int),
    "accspmm_spmm_chain": ([C.POINTER(METCF), vp, vp, u32, u32, i32, vp], C.c_int),
    "accspmm_gather_floor": ([C.POINTER(METCF), vp, u32, u32, i32, f32p, vp], C.c_int),
    "accspmm_spmm_host": ([C.POINTER(METCF), C.POINTER(ADPBME), vp, vp, u32, i32, vp], C.c_int),
    "accspmm_spmm_adaptive_noalloc": ([C.POINTER(ADPBME), vp, vp, u32, u32, i32, vp], C.c_int),
    "accspmm_noalloc_max_c_rows": ([], C.c_uint32),
    "accspmm_time_spmm": ([C.POINTER(METCF), C.POINTER(ADPBME), vp, vp, u32, u32, i32, i32, i32,
                           f32p, vp], C.c_int),
    "accspmm_set_option": ([i32, i32], C.c_int),
    "accspmm_get_option": ([i32, C.POINTER(i32)], C.c_int),
}

_LIB = None
_LAB = None


class AccSpmmError(RuntimeError):
    def __init__(self, fn: str, status: int, msg: str):
        super().__init__(f"{fn} returned {status}: {msg}")
        self.status = status


def header_functions() -> list:
    """Names of the functions declared in include/accspmm.h."""
    with open(HEADER) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(accspmm_\w+)\s*\(", text)))


def _open(path: str):
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


def load():
    """Loads libaccspmm.so; raises if it has not been built."""
    global _LIB
    if _LIB is None:
        _LIB = _open(LIB_PATH)
    return _LIB


def load_lab():
    """Loads the measurement build libaccspmm_lab.so (the same ABI with the
    variant kernels selectable through OPT_KERNEL, and accspmm_gather_floor);
    raises if it has not been built."""
    global _LAB
    if _LAB is None:
        _LAB = _open(LAB_PATH)
    return _LAB


def check(fn: str, status: int, lib=None) -> None:
    if status != SUCCESS:
        raise AccSpmmError(fn, status, (lib or load()).accspmm_last_error().decode())


def call(name: str, *args) -> None:
    check(name, getattr(load(), name)(*args))


def call_lab(name: str, *args) -> None:
    lab = load_lab()
    check(name, getattr(lab, name)(*args), lab)


def get_option(option: int, lib=None) -> int:
    v = C.c_int32()
    lib = lib or load()
    check("accspmm_get_option", lib.accspmm_get_option(option, C.byref(v)), lib)
    return v.value


def set_option(option: int, value: int, lib=None) -> None:
    lib = lib or load()
    check("accspmm_set_option", lib.accspmm_set_option(option, value), lib)


class option:
    """Context manager: an option set for the duration of a block, restored after.

        with capi.option(capi.OPT_PACK, 0):
            m.spmm(B, C, K)
    """

    def __init__(self, opt: int, value: int, lib=None):
        self.opt, self.value, self.lib = opt, value, lib

    def __enter__(self):
        self.old = get_option(self.opt, self.lib)
        set_option(self.opt, self.value, self.lib)
        return self

    def __exit__(self, *exc):
        set_option(self.opt, self.old, self.lib)
