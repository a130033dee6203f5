"""Host-side mirror of the reference's C++ interface over the C ABI.

The reference's calls (src/mma_tf32.cu) map one to one:
  read_from_mtx(path)              include/mmio.hpp:171   -> accspmm_read_mtx
  CSR(coo)                         include/format.hpp:110 -> accspmm_csr_from_coo
  METCFBit.convertFromCSR(csr)     include/format.hpp:215 -> accspmm_metcf_from_csr
  AdpBME.CSR2AdpBME(csr, 3, 1, 2)  include/format.hpp:340 -> accspmm_adpbme_from_metcf
  balanceStrategy(metcf)           include/utils.hpp:75   -> accspmm_balance_strategy
  TF32Compute.compute / adpBalanceCompute (include/tf32_comp.hpp:52, :82)
                                                          -> accspmm_spmm_tf32 / _adaptive
Host objects come back as numpy arrays; device objects stay library-owned
(freed by `destroy()` or garbage collection).  Dense device buffers are any
objects with a `data_ptr()` (torch tensors) or raw integer addresses.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import capi
from .capi import ADPBME, COO, CSR, METCF, call, load

_NP = {capi.u32p: np.uint32, capi.u64p: np.uint64, capi.f32p: np.float32}


def _arr(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array(ptr, (n,)).copy()


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def _addr(x) -> int:
    if x is None:
        return 0
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if isinstance(x, np.ndarray):
        return int(x.ctypes.data)
    return int(x)


def _stream(s) -> C.c_void_p:
    if s is None:
        return C.c_void_p(0)
    if hasattr(s, "cuda_stream"):
        return C.c_void_p(int(s.cuda_stream))
    return C.c_void_p(int(s))


# ---- host objects (numpy) ---------------------------------------------------

def read_from_mtx(path: str):
    """(status, coo dict) with the reference's return codes."""
    lib = load()
    coo = COO()
    st = lib.accspmm_read_mtx(path.encode(), C.byref(coo))
    if st != capi.SUCCESS:
        return st, None
    out = dict(rows=coo.rows, cols=coo.cols, nnz=coo.nnz, row=_arr(coo.row, coo.nnz, np.uint32),
               col=_arr(coo.col, coo.nnz, np.uint32), data=_arr(coo.data, coo.nnz, np.float32))
    lib.accspmm_coo_destroy(C.byref(coo))
    return st, out


class _Keep:
    """Keeps numpy arrays alive while a C struct points at them."""

    def __init__(self, struct, *arrays):
        self.struct = struct
        self.arrays = arrays


def coo_struct(rows, cols, row, col, data) -> _Keep:
    row = np.ascontiguousarray(row, np.uint32)
    col = np.ascontiguousarray(col, np.uint32)
    data = np.ascontiguousarray(data, np.float32)
    s = COO(rows, cols, len(row), _ptr(row, C.c_uint32), _ptr(col, C.c_uint32),
            _ptr(data, C.c_float), capi.HOST, 0)
    return _Keep(s, row, col, data)


def csr_struct(csr: dict) -> _Keep:
    rp = np.ascontiguousarray(csr["row_ptr"], np.uint32)
    ci = np.ascontiguousarray(csr["col_idx"], np.uint32)
    d = np.ascontiguousarray(csr["data"], np.float32)
    s = CSR(csr["rows"], csr["cols"], len(ci), _ptr(rp, C.c_uint32), _ptr(ci, C.c_uint32),
            _ptr(d, C.c_float), capi.HOST, 0)
    return _Keep(s, rp, ci, d)


def metcf_struct(m: dict) -> _Keep:
    rwo = np.ascontiguousarray(m["rwo"], np.uint32)
    tco = np.ascontiguousarray(m["tc_offset"], np.uint32)
    bits = np.ascontiguousarray(m["bits"], np.uint64)
    a2b = np.ascontiguousarray(m["a2b"], np.uint32)
    d = np.ascontiguousarray(m["data"], np.float32)
    s = METCF(m["rows"], m["cols"], m["nnz"], len(rwo) - 1, len(bits), _ptr(rwo, C.c_uint32),
              _ptr(tco, C.c_uint32), _ptr(bits, C.c_uint64), _ptr(a2b, C.c_uint32),
              _ptr(d, C.c_float), capi.HOST, 0)
    return _Keep(s, rwo, tco, bits, a2b, d)


def adpbme_struct(a: dict) -> _Keep:
    go = np.ascontiguousarray(a["group_offset"], np.uint32)
    tco = np.ascontiguousarray(a["tc_offset"], np.uint32)
    ri = np.ascontiguousarray(a["row_indices"], np.uint32)
    bits = np.ascontiguousarray(a["bits"], np.uint64)
    a2b = np.ascontiguousarray(a["a2b"], np.uint32)
    d = np.ascontiguousarray(a["data"], np.float32)
    s = ADPBME(a["rows"], a["cols"], a["nnz"], len(bits), len(go) - 1, _ptr(go, C.c_uint32),
               _ptr(tco, C.c_uint32), _ptr(ri, C.c_uint32), _ptr(bits, C.c_uint64),
               _ptr(a2b, C.c_uint32), _ptr(d, C.c_float), capi.HOST, 0)
    return _Keep(s, go, tco, ri, bits, a2b, d)


def csr_from_coo(rows, cols, row, col, data) -> dict:
    k = coo_struct(rows, cols, row, col, data)
    out = CSR()
    call("accspmm_csr_from_coo", C.byref(k.struct), C.byref(out), None)
    res = csr_to_numpy(out)
    load().accspmm_csr_destroy(C.byref(out))
    return res


def csr_to_numpy(c: CSR) -> dict:
    return dict(rows=c.rows, cols=c.cols, nnz=c.nnz,
                row_ptr=_arr(c.row_ptr, c.rows + 1, np.uint32),
                col_idx=_arr(c.col_idx, c.nnz, np.uint32), data=_arr(c.data, c.nnz, np.float32))


def metcf_to_numpy(m: METCF) -> dict:
    return dict(rows=m.rows, cols=m.cols, nnz=m.nnz,
                rwo=_arr(m.row_window_offset, m.num_windows + 1, np.uint32),
                tc_offset=_arr(m.tc_offset, m.num_tiles + 1, np.uint32),
                bits=_arr(m.tc_local_bit, m.num_tiles, np.uint64),
                a2b=_arr(m.sparse_a2b, 8 * m.num_tiles, np.uint32),
                data=_arr(m.data, m.nnz, np.float32))


def adpbme_to_numpy(a: ADPBME) -> dict:
    return dict(rows=a.rows, cols=a.cols, nnz=a.nnz,
                group_offset=_arr(a.group_offset, a.num_groups + 1, np.uint32),
                tc_offset=_arr(a.tc_offset, a.num_tiles + 1, np.uint32),
                row_indices=_arr(a.row_indices, a.num_tiles, np.uint32),
                bits=_arr(a.tc_local_bit, a.num_tiles, np.uint64),
                a2b=_arr(a.sparse_a2b, 8 * a.num_tiles, np.uint32),
                data=_arr(a.data, a.nnz, np.float32))


def metcf_from_csr(csr: dict) -> dict:
    k = csr_struct(csr)
    out = METCF()
    call("accspmm_metcf_from_csr", C.byref(k.struct), C.byref(out), None)
    res = metcf_to_numpy(out)
    load().accspmm_metcf_destroy(C.byref(out))
    return res


def adpbme_from_metcf(m: dict, t_load=3, t_comp=1, t_write=2, target_num=16) -> dict:
    k = metcf_struct(m)
    out = ADPBME()
    call("accspmm_adpbme_from_metcf", C.byref(k.struct), t_load, t_comp, t_write, target_num,
         C.byref(out), None)
    res = adpbme_to_numpy(out)
    load().accspmm_adpbme_destroy(C.byref(out))
    return res


def reorder_rcm(csr: dict):
    """Reverse Cuthill-McKee numbering of a square host CSR: (perm with
    perm[new] = old, bandwidth before, bandwidth after)."""
    k = csr_struct(csr)
    perm = np.empty(csr["rows"], np.uint32)
    b0, b1 = C.c_uint64(0), C.c_uint64(0)
    call("accspmm_reorder_rcm", C.byref(k.struct), _ptr(perm, C.c_uint32), C.byref(b0), C.byref(b1))
    return perm, int(b0.value), int(b1.value)


def csr_permute(csr: dict, perm) -> dict:
    """P A P^T of a square host CSR (A'[i, j] = A[perm[i], perm[j]])."""
    k = csr_struct(csr)
    p = np.ascontiguousarray(perm, np.uint32)
    out = CSR()
    call("accspmm_csr_permute", C.byref(k.struct), _ptr(p, C.c_uint32), C.byref(out))
    res = csr_to_numpy(out)
    load().accspmm_csr_destroy(C.byref(out))
    return res


def permute_rows(src, dst, idx, rows: int, K: int, scatter: bool = False, stream=None) -> None:
    """Device row gather dst[i] = src[idx[i]] (or scatter dst[idx[i]] = src[i])."""
    call("accspmm_dense_permute_rows", C.c_void_p(_addr(src)), C.c_void_p(_addr(dst)),
         C.c_void_p(_addr(idx)), rows, K, 1 if scatter else 0, _stream(stream))


def dense_matmul(H, n: int, k_in: int, W, k_out: int, XW, precision: int = capi.PREC_TF32,
                 stream=None) -> None:
    """XW = H W on the device (accspmm_dense_matmul): H n x k_in, W k_in x
    k_out, XW n x k_out, row-major fp32, on the tcgen05 tensor cores."""
    call("accspmm_dense_matmul", C.c_void_p(_addr(H)), n, k_in, C.c_void_p(_addr(W)), k_out,
         C.c_void_p(_addr(XW)), precision, _stream(stream))


def save_metcf(m: dict, path: str) -> None:
    """Writes a host METCF (dict of arrays) to a binary file."""
    k = metcf_struct(m)
    call("accspmm_metcf_save", C.byref(k.struct), os.fsencode(path), None)


def load_metcf(path: str) -> dict:
    """Reads and validates a binary METCF file into host arrays."""
    out = METCF()
    call("accspmm_metcf_load", os.fsencode(path), capi.HOST, C.byref(out), None)
    res = metcf_to_numpy(out)
    load().accspmm_metcf_destroy(C.byref(out))
    return res


def save_adpbme(a: dict, path: str) -> None:
    """Writes a host AdpBME (dict of arrays) to a binary file."""
    k = adpbme_struct(a)
    call("accspmm_adpbme_save", C.byref(k.struct), os.fsencode(path), None)


def load_adpbme(path: str) -> dict:
    """Reads and validates a binary AdpBME file into host arrays."""
    out = ADPBME()
    call("accspmm_adpbme_load", os.fsencode(path), capi.HOST, C.byref(out), None)
    res = adpbme_to_numpy(out)
    load().accspmm_adpbme_destroy(C.byref(out))
    return res


def balance_strategy(m: dict) -> int:
    k = metcf_struct(m)
    flag = C.c_int(-1)
    call("accspmm_balance_strategy", C.byref(k.struct), C.byref(flag), None)
    return flag.value


# ---- device objects -------------------------------------------------------------

class DeviceObject:
    """A library-owned device structure, destroyed when collected."""

    _destroy = None

    def __init__(self, struct):
        self.struct = struct

    def destroy(self):
        if self.struct is not None and self.struct.owned:
            if self.struct.space == capi.DEVICE:
                _sync_device()  # queued work may still read the arrays
            getattr(load(), self._destroy)(C.byref(self.struct))
        self.struct = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    @property
    def ref(self):
        return C.byref(self.struct)


class DeviceCOO(DeviceObject):
    _destroy = "accspmm_coo_destroy"


class DeviceCSR(DeviceObject):
    _destroy = "accspmm_csr_destroy"

    @classmethod
    def upload(cls, csr: dict, stream=None) -> "DeviceCSR":
        k = csr_struct(csr)
        out = CSR()
        call("accspmm_csr_copy", C.byref(k.struct), capi.DEVICE, C.byref(out), _stream(stream))
        _sync(stream)
        return cls(out)


class DeviceMETCF(DeviceObject):
    _destroy = "accspmm_metcf_destroy"

    @classmethod
    def upload(cls, m: dict, stream=None) -> "DeviceMETCF":
        k = metcf_struct(m)
        out = METCF()
        call("accspmm_metcf_copy", C.byref(k.struct), capi.DEVICE, C.byref(out), _stream(stream))
        _sync(stream)
        return cls(out)

    @classmethod
    def load(cls, path: str, stream=None) -> "DeviceMETCF":
        """Reads and validates a binary METCF file straight into device memory."""
        out = METCF()
        call("accspmm_metcf_load", os.fsencode(path), capi.DEVICE, C.byref(out), _stream(stream))
        return cls(out)

    def save(self, path: str, stream=None) -> None:
        call("accspmm_metcf_save", self.ref, os.fsencode(path), _stream(stream))

    @classmethod
    def from_csr(cls, dcsr: DeviceCSR, stream=None) -> "DeviceMETCF":
        out = METCF()
        call("accspmm_metcf_from_csr", dcsr.ref, C.byref(out), _stream(stream))
        return cls(out)

    def to_numpy(self, stream=None) -> dict:
        h = METCF()
        call("accspmm_metcf_copy", self.ref, capi.HOST, C.byref(h), _stream(stream))
        res = metcf_to_numpy(h)
        load().accspmm_metcf_destroy(C.byref(h))
        return res

    @property
    def c_rows(self) -> int:
        return 8 * self.struct.num_windows

    def balance_strategy(self, stream=None) -> int:
        flag = C.c_int(-1)
        call("accspmm_balance_strategy", self.ref, C.byref(flag), _stream(stream))
        return flag.value

    def adpbme(self, t_load=3, t_comp=1, t_write=2, target_num=16, stream=None) -> "DeviceADPBME":
        out = ADPBME()
        call("accspmm_adpbme_from_metcf", self.ref, t_load, t_comp, t_write, target_num,
             C.byref(out), _stream(stream))
        return DeviceADPBME(out)

    def spmm(self, B, C_out, K: int, precision: int = capi.PREC_TF32, stream=None) -> None:
        call("accspmm_spmm_tf32", self.ref, C.c_void_p(_addr(B)), C.c_void_p(_addr(C_out)), K,
             precision, _stream(stream))

    def matmul(self, B, precision: int = capi.PREC_TF32):
        """A @ B for a CUDA float32 tensor B of cols x K (K a multiple of 4):
        a new tensor of rows x K, computed on torch's current stream (a view
        of the 8 * num_windows rows the kernel writes)."""
        import torch
        if B.dim() != 2 or B.shape[0] != self.struct.cols or B.dtype != torch.float32 or not B.is_cuda:
            raise ValueError(f"B must be a CUDA float32 tensor of {self.struct.cols} rows")
        B = B.contiguous()
        K = int(B.shape[1])
        out = torch.empty((self.c_rows, K), device=B.device, dtype=torch.float32)
        self.spmm(B, out, K, precision, torch.cuda.current_stream(B.device))
        return out[: self.struct.rows]

    def spmm_bias_act(self, B, C_out, K: int, bias=None, activation: int = capi.ACT_NONE,
                      precision: int = capi.PREC_TF32, stream=None) -> None:
        """C_out = act(A * B + bias) with the epilogue fused into the C store."""
        call("accspmm_spmm_bias_act", self.ref, C.c_void_p(_addr(B)), C.c_void_p(_addr(C_out)), K,
             precision, C.c_void_p(_addr(bias)), activation, _stream(stream))

    def spmm_chain(self, B, C_out, K: int, hops: int = 2, precision: int = capi.PREC_TF32,
                   stream=None) -> None:
        """C_out = A^hops * B on the device (accspmm_spmm_chain)."""
        call("accspmm_spmm_chain", self.ref, C.c_void_p(_addr(B)), C.c_void_p(_addr(C_out)), K,
             hops, precision, _stream(stream))

    def gather_floor(self, B, K: int, repeats: int = 10, stream=None, slice_width: int = 0) -> float:
        """Milliseconds of a launch that only gathers the B rows this SpMM
        reads (accspmm_gather_floor of the measurement build,
        libaccspmm_lab.so), in the SpMM's launch shape or in the
        register-direct shape of another slice width."""
        ms = C.c_float(0.0)
        capi.call_lab("accspmm_gather_floor", self.ref, C.c_void_p(_addr(B)), K, slice_width, repeats,
                      C.byref(ms), _stream(stream))
        return float(ms.value)

    def gcn_layer(self, H, k_in: int, W, k_out: int, out, bias=None,
                  activation: int = capi.ACT_RELU, precision: int = capi.PREC_TF32,
                  stream=None) -> None:
        """out = act(A * (H W) + bias): the tcgen05 GEMM for H W, the fused
        SpMM for A."""
        call("accspmm_gcn_layer", self.ref, C.c_void_p(_addr(H)), k_in, C.c_void_p(_addr(W)),
             k_out, C.c_void_p(_addr(bias)), activation, C.c_void_p(_addr(out)), precision,
             _stream(stream))

    def spmm_host(self, B_host, C_host, K: int, precision: int = capi.PREC_TF32, stream=None) -> None:
        """C_host = A * B_host with both dense matrices in host memory
        (accspmm_spmm_host); C_host has 8 ceil(rows / 8) rows.  Complete when
        `stream` is."""
        call("accspmm_spmm_host", self.ref, None, C.c_void_p(_addr(B_host)),
             C.c_void_p(_addr(C_host)), K, precision, _stream(stream))

    def autotune(self, B, C_out, K: int, precision: int = capi.PREC_TF32, stream=None) -> dict:
        """Times the candidate launch shapes and keeps the fastest for this
        matrix's signature (overwrites C_out)."""
        r = capi.TUNE()
        call("accspmm_autotune_metcf", self.ref, C.c_void_p(_addr(B)), C.c_void_p(_addr(C_out)),
             K, precision, _stream(stream), C.byref(r))
        return dict(kernel={0: "direct", 4: "double-buffered"}.get(r.kernel, str(r.kernel)),
                    slice_width=r.slice_width, windows_per_cta=r.windows_per_cta,
                    ctas_per_sm=r.ctas_per_sm, tile_ring=r.tile_ring, packed_b=r.packed_b, best_ms=round(r.best_ms, 4),
                    default_ms=round(r.default_ms, 4), candidates=r.candidates)


class DeviceADPBME(DeviceObject):
    _destroy = "accspmm_adpbme_destroy"

    def to_numpy(self, stream=None) -> dict:
        h = ADPBME()
        call("accspmm_adpbme_copy", self.ref, capi.HOST, C.byref(h), _stream(stream))
        res = adpbme_to_numpy(h)
        load().accspmm_adpbme_destroy(C.byref(h))
        return res

    def c_rows(self, stream=None) -> int:
        v = C.c_uint32(0)
        call("accspmm_adaptive_c_rows", self.ref, C.byref(v), _stream(stream))
        return v.value

    def spmm_host(self, B_host, C_host, K: int, precision: int = capi.PREC_TF32, stream=None) -> None:
        """Adaptive-path C_host = A * B_host from host memory
        (accspmm_spmm_host); C_host has 8 ceil(rows / 8) rows."""
        call("accspmm_spmm_host", None, self.ref, C.c_void_p(_addr(B_host)),
             C.c_void_p(_addr(C_host)), K, precision, _stream(stream))

    def spmm(self, B, C_out, c_rows: int, K: int, precision: int = capi.PREC_TF32,
             stream=None) -> None:
        call("accspmm_spmm_adaptive", self.ref, C.c_void_p(_addr(B)), C.c_void_p(_addr(C_out)),
             c_rows, K, precision, _stream(stream))


class Batch:
    """A batch plan: many device METCF matrices in one persistent launch.

    items: list of (DeviceMETCF, B, C, K); B and C must stay allocated and in
    place for the plan's lifetime."""

    def __init__(self, items, precision=capi.PREC_TF32):
        arr = (capi.BATCHITEM * len(items))()
        for i, (m, B, C_out, K) in enumerate(items):
            arr[i].metcf = C.pointer(m.struct)
            arr[i].B = C.c_void_p(_addr(B))
            arr[i].C = C.c_void_p(_addr(C_out))
            arr[i].K = K
        self._keep = [it[0] for it in items]
        h = C.c_void_p()
        call("accspmm_batch_create", arr, len(items), precision, C.byref(h))
        self.h = h

    def run(self, stream=None):
        call("accspmm_batch_run", self.h, _stream(stream))

    def capture(self, stream):
        call("accspmm_batch_capture", self.h, _stream(stream))

    def launch_graph(self, stream):
        call("accspmm_batch_launch_graph", self.h, _stream(stream))

    def info(self):
        n, w, fs = C.c_uint32(), C.c_uint32(), C.c_uint32()
        call("accspmm_batch_info", self.h, C.byref(n), C.byref(w), C.byref(fs))
        return n.value, w.value, fs.value

    def destroy(self):
        if self.h:
            load().accspmm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Server:
    """Continuous-batching request server over resident device METCF graphs.

    Host B / C buffers (torch pinned tensors or raw addresses) must stay
    valid until wait() returns for their request."""

    def __init__(self, graphs, hbm_budget_bytes, max_batch=64, streams=4):
        arr = (METCF * len(graphs))()
        for i, g in enumerate(graphs):
            arr[i] = g.struct
        self._keep = list(graphs)
        cfg = capi.SERVERCFG(hbm_budget_bytes, max_batch, streams)
        h = C.c_void_p()
        call("accspmm_server_create", arr, len(graphs), C.byref(cfg), C.byref(h))
        self.h = h

    def submit(self, graph: int, B_host, C_host, K: int, precision=capi.PREC_TF32, chain=1) -> int:
        rid = C.c_uint64()
        call("accspmm_server_submit", self.h, graph, C.c_void_p(_addr(B_host)),
             C.c_void_p(_addr(C_host)), K, precision, chain, C.byref(rid))
        return rid.value

    def wait(self, rid: int, timeout_ms: int = -1) -> int:
        """Returns the request's status (0 on success)."""
        return load().accspmm_server_wait(self.h, rid, timeout_ms)

    def cancel(self, rid: int) -> int:
        return load().accspmm_server_cancel(self.h, rid)

    def stats(self) -> dict:
        st = capi.SERVERSTATS()
        call("accspmm_server_stats", self.h, C.byref(st))
        return {k: getattr(st, k) for k, _ in capi.SERVERSTATS._fields_}

    def reset_stats(self):
        call("accspmm_server_reset_stats", self.h)

    def destroy(self):
        if self.h:
            load().accspmm_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def time_spmm(metcf: DeviceMETCF | None, adp: DeviceADPBME | None, B, C_out, c_rows: int, K: int,
              precision=capi.PREC_TF32, warmup=10, exe=10, stream=None) -> float:
    """TF32Compute's timing loop (include/tf32_comp.hpp:33-46): average ms."""
    ms = C.c_float(0)
    call("accspmm_time_spmm", metcf.ref if metcf else None, adp.ref if adp else None,
         C.c_void_p(_addr(B)), C.c_void_p(_addr(C_out)), c_rows, K, precision, warmup, exe,
         C.byref(ms), _stream(stream))
    return ms.value


def _sync_device():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except ImportError:
        pass


def _sync(stream):
    try:
        import torch
        if torch.cuda.is_available():
            (stream or torch.cuda.current_stream()).synchronize()
    except ImportError:
        pass
