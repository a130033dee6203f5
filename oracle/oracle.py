"""ctypes binding of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: imported by the tests, by the smoke check and by the
CPU-baseline leg of bench.py, always as the checker or the timed CPU
baseline, never as the product path.  `load()` builds liboracle.so with make
when it is missing.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return os.path.join(HERE, "liboracle.so")


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    path = os.path.join(HERE, "liboracle.so")
    src = os.path.join(HERE, "oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        build()
    lib = C.CDLL(path)
    lib.oracle_read_mtx.argtypes = [C.c_char_p] + [C.POINTER(C.c_uint32)] * 3 + [
        C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.POINTER(C.c_uint32)),
        C.POINTER(C.POINTER(C.c_float))]
    lib.oracle_read_mtx.restype = C.c_int
    lib.oracle_free.argtypes = [C.c_void_p]
    lib.oracle_csr_from_coo.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, f32p,
                                        u32p, u32p, f32p]
    lib.oracle_metcf_num_tiles.argtypes = [C.c_uint32, u32p, u32p]
    lib.oracle_metcf_num_tiles.restype = C.c_uint64
    lib.oracle_metcf_fill.argtypes = [C.c_uint32, u32p, u32p, f32p, u32p, u32p,
                                      u64p, u32p, f32p]
    lib.oracle_adpbme_groups.argtypes = [C.c_uint32, u32p] + [C.c_uint32] * 4 + [C.c_void_p]
    lib.oracle_adpbme_groups.restype = C.c_uint32
    lib.oracle_adpbme_row_indices.argtypes = [C.c_uint32, u32p, u32p]
    lib.oracle_balance_strategy.argtypes = [u32p, C.c_uint32, C.c_uint32]
    lib.oracle_balance_strategy.restype = C.c_int
    lib.oracle_tf32_rna.argtypes = [C.c_float]
    lib.oracle_tf32_rna.restype = C.c_float
    lib.oracle_spmm_metcf_f64.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, u64p,
                                          u32p, f32p, f32p, C.c_uint32, f64p]
    lib.oracle_spmm_metcf_tf32.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, u64p,
                                           u32p, f32p, f32p, C.c_uint32, f32p]
    lib.oracle_spmm_csr_f64.argtypes = [C.c_uint32, u32p, u32p, f32p, f32p,
                                        C.c_uint32, f64p]
    lib.oracle_spmm_csr_f32_omp.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, f32p,
                                            f32p, C.c_uint32, f32p, C.c_int]
    lib.oracle_omp_max_threads.restype = C.c_int
    _LIB = lib
    return lib


def read_mtx(path: str):
    """Returns (status, dict) like include/mmio.hpp:171 read_from_mtx."""
    lib = load()
    rows, cols, nnz = C.c_uint32(), C.c_uint32(), C.c_uint32()
    r, c, d = C.POINTER(C.c_uint32)(), C.POINTER(C.c_uint32)(), C.POINTER(C.c_float)()
    st = lib.oracle_read_mtx(path.encode(), C.byref(rows), C.byref(cols), C.byref(nnz),
                             C.byref(r), C.byref(c), C.byref(d))
    if st != 0:
        return st, None
    n = nnz.value
    out = dict(rows=rows.value, cols=cols.value, nnz=n,
               row=np.ctypeslib.as_array(r, (n,)).copy() if n else np.zeros(0, np.uint32),
               col=np.ctypeslib.as_array(c, (n,)).copy() if n else np.zeros(0, np.uint32),
               data=np.ctypeslib.as_array(d, (n,)).copy() if n else np.zeros(0, np.float32))
    for p in (r, c, d):
        lib.oracle_free(C.cast(p, C.c_void_p))
    return st, out


def csr_from_coo(rows: int, row, col, data):
    lib = load()
    row = np.ascontiguousarray(row, np.uint32)
    col = np.ascontiguousarray(col, np.uint32)
    data = np.ascontiguousarray(data, np.float32)
    rp = np.zeros(rows + 1, np.uint32)
    ci = np.zeros(len(col), np.uint32)
    v = np.zeros(len(col), np.float32)
    lib.oracle_csr_from_coo(rows, len(col), row, col, data, rp, ci, v)
    return rp, ci, v


def metcf(rows: int, row_ptr, col_idx, vals) -> dict:
    """include/format.hpp:215-274 restated; returns the five METCF arrays."""
    lib = load()
    row_ptr = np.ascontiguousarray(row_ptr, np.uint32)
    col_idx = np.ascontiguousarray(col_idx, np.uint32)
    vals = np.ascontiguousarray(vals, np.float32)
    t = int(lib.oracle_metcf_num_tiles(rows, row_ptr, col_idx))
    w = (rows + 7) // 8
    out = dict(rwo=np.zeros(w + 1, np.uint32), tc_offset=np.zeros(t + 1, np.uint32),
               bits=np.zeros(t, np.uint64), a2b=np.zeros(8 * t, np.uint32),
               data=np.zeros(len(vals), np.float32))
    lib.oracle_metcf_fill(rows, row_ptr, col_idx, vals, out["rwo"], out["tc_offset"],
                          out["bits"], out["a2b"], out["data"])
    return out


def adpbme_groups(rwo, t_load=3, t_comp=1, t_write=2, target_num=16):
    lib = load()
    rwo = np.ascontiguousarray(rwo, np.uint32)
    w = len(rwo) - 1
    g = lib.oracle_adpbme_groups(w, rwo, t_load, t_comp, t_write, target_num, None)
    go = np.zeros(g + 1, np.uint32)
    lib.oracle_adpbme_groups(w, rwo, t_load, t_comp, t_write, target_num,
                             go.ctypes.data_as(C.c_void_p))
    return go


def adpbme_row_indices(rwo):
    lib = load()
    rwo = np.ascontiguousarray(rwo, np.uint32)
    ri = np.zeros(int(rwo[-1]), np.uint32)
    lib.oracle_adpbme_row_indices(len(rwo) - 1, rwo, ri)
    return ri


def balance_strategy(rwo) -> int:
    lib = load()
    rwo = np.ascontiguousarray(rwo, np.uint32)
    return int(lib.oracle_balance_strategy(rwo, len(rwo) - 1, int(rwo[-1])))


def tf32_rna(x: float) -> float:
    return float(load().oracle_tf32_rna(x))


def spmm_metcf_f64(m: dict, cols: int, B: np.ndarray) -> np.ndarray:
    lib = load()
    B = np.ascontiguousarray(B, np.float32)
    k = B.shape[1]
    w = len(m["rwo"]) - 1
    out = np.zeros((8 * w, k), np.float64)
    lib.oracle_spmm_metcf_f64(w, cols, m["rwo"], m["tc_offset"], m["bits"], m["a2b"],
                              m["data"], B, k, out)
    return out


def spmm_metcf_tf32(m: dict, cols: int, B: np.ndarray) -> np.ndarray:
    lib = load()
    B = np.ascontiguousarray(B, np.float32)
    k = B.shape[1]
    w = len(m["rwo"]) - 1
    out = np.zeros((8 * w, k), np.float32)
    lib.oracle_spmm_metcf_tf32(w, cols, m["rwo"], m["tc_offset"], m["bits"], m["a2b"],
                               m["data"], B, k, out)
    return out


def spmm_csr_f64(row_ptr, col_idx, vals, B) -> np.ndarray:
    lib = load()
    B = np.ascontiguousarray(B, np.float32)
    rows = len(row_ptr) - 1
    out = np.zeros((rows, B.shape[1]), np.float64)
    lib.oracle_spmm_csr_f64(rows, np.ascontiguousarray(row_ptr, np.uint32),
                            np.ascontiguousarray(col_idx, np.uint32),
                            np.ascontiguousarray(vals, np.float32), B, B.shape[1], out)
    return out


def spmm_csr_f32_omp(row_ptr, col_idx, vals, B, C_out, row_begin=0, row_end=None,
                     threads=0):
    """CPU baseline: FP32 CSR SpMM on `threads` OpenMP threads (0 = all)."""
    lib = load()
    rows = len(row_ptr) - 1
    if row_end is None:
        row_end = rows
    lib.oracle_spmm_csr_f32_omp(row_begin, row_end, row_ptr, col_idx, vals, B,
                                B.shape[1], C_out, threads)
    return C_out


def omp_max_threads() -> int:
    return int(load().oracle_omp_max_threads())
