"""The reference's own SpMM kernels, timed on the GPU (measurement only).

MEASUREMENT INFRASTRUCTURE, like the rest of oracle/: used by the reference
arm of bench.py to put the reference's kernels on the same GPU beside the
product, never by the product path.

`oracle/_ref/ref_kernels.cubin` is include/mma_tf32.cuh of the reference,
compiled for sm_103a from its sources by `make -C oracle refkernels` (the
sources are never copied).  This module loads it through the CUDA driver API
and times its kernels the way the reference's driver does:
  - kernel and block choice of TF32Compute (include/tf32_comp.hpp:19-31,
    52-111): the plain path launches tf32_mma_kernel (K <= 512) on a grid of
    W windows, the adaptive path tf32_mma_balance_kernel (K <= 128) or
    tf32_mma_balance_g128_kernel (K > 128) on a grid of G groups; blocks of
    32 x K/32 threads up to the threshold (512 plain, 128 adaptive,
    src/mma_tf32.cu:218), 32 x K/64 above it;
  - numNodes = the matrix's rows (src/mma_tf32.cu:208), C of 8W rows (plain)
    or max(8G, rowIndices.back() + 8) rows (adaptive, src/mma_tf32.cu:112),
    zeroed once before the launches as the reference's driver does;
  - 10 warm-up launches, then 10 launches between two events on the legacy
    default stream, average per launch (include/tf32_comp.hpp:33-46).

Bounds, read from include/mma_tf32.cuh: every B load is of a sparseA2B entry
that is not greater than numNodes (padding entries are UINT32_MAX and are
skipped), at columns below K; C stores and atomics stay in the C rows above.
Three reads can pass the end of an array by a few elements: the first tile of
a trailing empty window (tcLocalBit[T], sparseA2B[8T .. 8T + 7], plain
kernel), the prefetch of a one-tile last group's second tile
(sparseA2B[8T .. 8T + 15], rowIndices[T], balance kernel).  Every array is
therefore uploaded with 64 elements of slack (padding value for sparseA2B),
so all of them land inside the buffers.  The kernels' results are not used
here (they are wrong for general B, src/mma_tf32.cu defects: tile 0's indices
for every window's first tile, the balance kernels' warps re-reading columns
0-31 or 0-63); only their time is.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")
PAD = 0xFFFFFFFF
SLACK = 64


def available() -> str | None:
    """None when the kernels can be timed here, else the reason."""
    if not os.path.exists(CUBIN):
        return "oracle/_ref/ref_kernels.cubin not built (make -C oracle refkernels where the reference sources are)"
    try:
        import torch
    except ImportError:
        return "torch is not importable"
    if not torch.cuda.is_available():
        return "no GPU"
    return None


def _check(r, what):
    if r != 0:
        raise RuntimeError(f"{what} failed with CUDA driver error {r}")


class RefKernels:
    """The reference's SpMM kernels loaded from the cubin."""

    NAMES = ("tf32_mma_kernel", "tf32_mma_balance_kernel", "tf32_mma_balance_g128_kernel")

    def __init__(self):
        import torch
        torch.zeros(1, device="cuda")  # makes the primary context current
        self.cu = C.CDLL("libcuda.so.1")
        _check(self.cu.cuInit(0), "cuInit")
        self.mod = C.c_void_p()
        _check(self.cu.cuModuleLoad(C.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        for n in self.NAMES:
            f = C.c_void_p()
            _check(self.cu.cuModuleGetFunction(C.byref(f), self.mod, n.encode()), f"cuModuleGetFunction({n})")
            self.fn[n] = f

    def _time(self, fn, grid, block, args, warmup=10, reps=10) -> float:
        cu = self.cu
        params = (C.c_void_p * len(args))(*[C.cast(C.byref(a), C.c_void_p) for a in args])
        e0, e1 = C.c_void_p(), C.c_void_p()
        _check(cu.cuEventCreate(C.byref(e0), 0), "cuEventCreate")
        _check(cu.cuEventCreate(C.byref(e1), 0), "cuEventCreate")
        try:
            for _ in range(warmup):
                _check(cu.cuLaunchKernel(fn, grid, 1, 1, block[0], block[1], 1, 0, None, params, None),
                       "cuLaunchKernel")
            _check(cu.cuCtxSynchronize(), "cuCtxSynchronize")
            _check(cu.cuEventRecord(e0, None), "cuEventRecord")
            for _ in range(reps):
                _check(cu.cuLaunchKernel(fn, grid, 1, 1, block[0], block[1], 1, 0, None, params, None),
                       "cuLaunchKernel")
            _check(cu.cuEventRecord(e1, None), "cuEventRecord")
            _check(cu.cuEventSynchronize(e1), "cuEventSynchronize")
            ms = C.c_float()
            _check(cu.cuEventElapsedTime(C.byref(ms), e0, e1), "cuEventElapsedTime")
            _check(cu.cuCtxSynchronize(), "cuCtxSynchronize")
        finally:
            cu.cuEventDestroy_v2(e0)
            cu.cuEventDestroy_v2(e1)
        return ms.value / reps


def _upload(a: np.ndarray, pad_value=0):
    """Device copy of a with SLACK trailing elements of pad_value."""
    import torch
    signed = {np.dtype(np.uint64): np.int64, np.dtype(np.uint32): np.int32, np.dtype(np.float32): np.float32}
    ext = np.full(len(a) + SLACK, pad_value, dtype=a.dtype)
    ext[:len(a)] = a
    return torch.from_numpy(ext.view(signed[a.dtype])).cuda()


def launch_config(K: int, adaptive: bool, W: int, G: int | None = None):
    """(kernel name, grid, block) the reference's driver uses: TF32Compute
    with threshold 512 on the plain path and 128 on the adaptive path
    (src/mma_tf32.cu:218, include/tf32_comp.hpp:19-31, 52-111)."""
    threshold = 128 if adaptive else 512
    warps = K // 32 if K <= threshold else K // 64
    if adaptive:
        name = "tf32_mma_balance_kernel" if K <= threshold else "tf32_mma_balance_g128_kernel"
        return name, int(G), (32, warps)
    name = "tf32_mma_kernel" if K <= threshold else "tf32_mma_g512_kernel"
    return name, int(W), (32, warps)


def time_reference_path(m: dict, rows: int, B, K: int, adaptive: bool, groups=None, row_indices=None,
                        kernels: RefKernels | None = None) -> dict:
    """Average ms per launch of the kernel the reference's driver runs for
    this matrix and K; m is the METCF dict of oracle.metcf (square matrix,
    rows = cols), B a CUDA float32 tensor of rows x K."""
    import torch
    assert B.is_cuda and B.dtype == torch.float32 and tuple(B.shape) == (rows, K) and B.is_contiguous()
    assert K % 32 == 0 and 32 <= K <= 512 and rows * K < 2 ** 32  # tf32_mma_g512_kernel not loaded
    a2b = m["a2b"]
    assert ((a2b < rows) | (a2b == PAD)).all()
    ker = kernels or RefKernels()
    W = len(m["rwo"]) - 1
    d = {"bits": _upload(m["bits"]), "a2b": _upload(a2b, PAD), "data": _upload(m["data"]),
         "rwo": _upload(m["rwo"], m["rwo"][-1]), "tco": _upload(m["tc_offset"], m["tc_offset"][-1])}
    p = lambda t: C.c_uint64(t.data_ptr())  # noqa: E731
    Bp = C.c_uint64(B.data_ptr())
    if not adaptive:
        name, grid, block = launch_config(K, False, W)
        Cd = torch.zeros((8 * W + 8, K), device="cuda")
        args = [p(d["bits"]), p(d["a2b"]), p(d["data"]), p(d["rwo"]), p(d["tco"]), Bp, p(Cd),
                C.c_uint32(rows), C.c_uint32(K)]
    else:
        assert groups is not None and row_indices is not None and len(groups) >= 2
        G = len(groups) - 1
        name, grid, block = launch_config(K, True, W, G)
        c_rows = max(8 * G, int(row_indices[-1]) + 8)
        Cd = torch.zeros((c_rows + 8, K), device="cuda")
        go = _upload(groups, groups[-1])
        ri = _upload(row_indices, row_indices[-1])
        args = [p(go), p(d["tco"]), p(ri), p(d["bits"]), p(d["a2b"]), p(d["data"]), Bp, p(Cd),
                C.c_uint32(rows), C.c_uint32(K)]
    torch.cuda.synchronize()
    ms = ker._time(ker.fn[name], grid, block, args)
    torch.cuda.synchronize()
    return {"kernel": name, "grid": int(grid), "block": list(block), "ms": round(ms, 4)}
