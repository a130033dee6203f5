"""Golden SpMM outputs of the reference's own GPU kernel.

Runs the reference's tf32_mma_kernel (include/mma_tf32.cuh:13-228), compiled
from the reference sources into oracle/_ref/ref_kernels.cubin by
`make -C oracle refkernels`, on a GPU, and saves what it writes:
tests/golden/ref_spmm/<case>_k<K>.npz with the dense B vector v and C.

The kernel is launched once with the reference's own configuration (grid W,
block 32 x K/32, include/tf32_comp.hpp:19-31, 52-80) on the reference's METCF
arrays of each golden case (the m_* arrays of <case>.npz, which came from the
reference's host code).  Inputs are restricted to those on which the
reference kernel computes the product A*B, because of its indexing:
  - for the first tile of every window it reads B rows through the first 8
    sparseA2B entries of the whole matrix (include/mma_tf32.cuh:92-93), so B
    has identical rows (every row equals v) and tile 0 holds 8 real columns
    (no padding there to zero a term);
  - an empty window would read the next window's first tile, so every window
    holds a tile;
  - at K < 64 the 64 tile values are not all staged (tid < 64 with K threads),
    so K is 64 or 128;
  - a sparseA2B entry counts as padding when it is greater than the kernel's
    numNodes argument (:94, :103), so numNodes = cols - 1 here: every real
    column is < cols and is loaded, padding (UINT32_MAX) is not, and no load
    reaches past B's last row (for the square cases this treats entries
    exactly as the reference driver's numNodes = rows does).
The adaptive path is pinned the same way: tf32_mma_balance_kernel
(include/mma_tf32.cuh:552-792), launched once on a zeroed C of
max(8G, rowIndices.back() + 8) rows (src/mma_tf32.cu:112) with the
reference's AdpBME arrays (the a_* arrays, parameters 3, 1, 2, 16), grid G,
block 32 x K/32 (include/tf32_comp.hpp:19-31 with threshold 128), writes
<case>_adp_k<K>.npz with B0 and C.  That kernel computes A*B when B's columns
repeat with period 16, B = tile(B0, K / 16) for any B0 of cols x 16: every warp
reads columns 0-31 (colB02 = groupID, no warp offset, :586-587) and the last
tile of a group uses the columns 16-31 fragment for columns 0-15 too (:779-780);
rows may differ (it reads each group's own sparseA2B).  Its arrays are uploaded
with 64 elements of slack, because the prefetch of a one-tile last group's
second tile reads sparseA2B[8T .. 8T + 15] and rowIndices[T] (:610, :623-624).
Not run by the tests: it needs a GPU and the cubin, whose source exists only
where the reference is checked out.  Run it as
    python tests/golden/make_ref_spmm.py [--adaptive] [--out DIR]
on a GPU machine with the cubin present; it needs torch (device memory) and
the CUDA driver library.  The .npz files go to DIR (default: ref_spmm/ in
this folder).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_kernels.cubin")
CASES = ["rand203", "longwin", "plsym1000"]
KS = [64, 128]
PAD = 0xFFFFFFFF


def check(r, what):
    if r != 0:
        raise RuntimeError(f"{what} failed with CUDA driver error {r}")


def main() -> int:
    import torch

    out_dir = sys.argv[sys.argv.index("--out") + 1] if "--out" in sys.argv else os.path.join(HERE, "ref_spmm")
    os.makedirs(out_dir, exist_ok=True)
    torch.cuda.init()
    torch.zeros(1, device="cuda")  # makes the primary context current
    cu = C.CDLL("libcuda.so.1")
    check(cu.cuInit(0), "cuInit")
    mod = C.c_void_p()
    check(cu.cuModuleLoad(C.byref(mod), CUBIN.encode()), "cuModuleLoad")
    fn = C.c_void_p()
    check(cu.cuModuleGetFunction(C.byref(fn), mod, b"tf32_mma_kernel"), "cuModuleGetFunction")
    rng = np.random.default_rng(2024)
    for case in CASES:
        g = dict(np.load(os.path.join(HERE, case + ".npz")))
        n_cols = int(g["dims"][1])
        rwo, a2b = g["m_rwo"], g["m_a2b"]
        W = len(rwo) - 1
        assert (rwo[1:] > rwo[:-1]).all(), f"{case}: an empty window"
        assert (a2b[:8] != PAD).all(), f"{case}: padding in tile 0"
        signed = {np.dtype(np.uint64): np.int64, np.dtype(np.uint32): np.int32,
                  np.dtype(np.float32): np.float32}
        dev = {k: torch.from_numpy(np.ascontiguousarray(g[k]).view(signed[g[k].dtype])).cuda()
               for k in ("m_bits", "m_a2b", "m_data", "m_rwo", "m_tc_offset")}
        for K in KS:
            assert n_cols * K < 2 ** 32 and K % 32 == 0 and 64 <= K <= 512
            v = rng.uniform(-1, 1, K).astype(np.float32)
            B = torch.from_numpy(np.tile(v, (n_cols, 1))).cuda()
            Cd = torch.full((8 * W, K), float("nan"), device="cuda")
            args = [C.c_uint64(dev["m_bits"].data_ptr()), C.c_uint64(dev["m_a2b"].data_ptr()),
                    C.c_uint64(dev["m_data"].data_ptr()), C.c_uint64(dev["m_rwo"].data_ptr()),
                    C.c_uint64(dev["m_tc_offset"].data_ptr()), C.c_uint64(B.data_ptr()),
                    C.c_uint64(Cd.data_ptr()), C.c_uint32(n_cols - 1), C.c_uint32(K)]
            params = (C.c_void_p * len(args))(*[C.cast(C.byref(a), C.c_void_p) for a in args])
            torch.cuda.synchronize()
            check(cu.cuLaunchKernel(fn, W, 1, 1, 32, K // 32, 1, 0, None, params, None), "cuLaunchKernel")
            check(cu.cuCtxSynchronize(), "cuCtxSynchronize")
            out = Cd.cpu().numpy()
            path = os.path.join(out_dir, f"{case}_k{K}.npz")
            np.savez_compressed(path, v=v, C=out, K=np.array([K], np.int32))
            print(f"{case} K={K}: C {out.shape}, finite {np.isfinite(out).all()} -> {path}")
    return 0


ADP_CASES = ["rand203", "longwin", "plsym1000", "ragged_unsorted"]


def slack(torch, a, pad_value):
    """Device copy of a with 64 trailing elements of pad_value."""
    signed = {np.dtype(np.uint64): np.int64, np.dtype(np.uint32): np.int32,
              np.dtype(np.float32): np.float32}
    ext = np.full(len(a) + 64, pad_value, dtype=a.dtype)
    ext[:len(a)] = a
    return torch.from_numpy(ext.view(signed[a.dtype])).cuda()


def main_adaptive(out_dir: str) -> int:
    import torch

    torch.cuda.init()
    torch.zeros(1, device="cuda")
    cu = C.CDLL("libcuda.so.1")
    check(cu.cuInit(0), "cuInit")
    mod = C.c_void_p()
    check(cu.cuModuleLoad(C.byref(mod), CUBIN.encode()), "cuModuleLoad")
    fn = C.c_void_p()
    check(cu.cuModuleGetFunction(C.byref(fn), mod, b"tf32_mma_balance_kernel"), "cuModuleGetFunction")
    rng = np.random.default_rng(2025)
    for case in ADP_CASES:
        g = dict(np.load(os.path.join(HERE, case + ".npz")))
        n_cols = int(g["dims"][1])
        go, ri = g["a_group_offset"], g["a_row_indices"]
        G = len(go) - 1
        assert G >= 1 and len(ri) >= 1
        c_rows = max(8 * G, int(ri[-1]) + 8)
        dev = {"go": slack(torch, go, go[-1]), "tco": slack(torch, g["a_tc_offset"], g["a_tc_offset"][-1]),
               "ri": slack(torch, ri, ri[-1]), "bits": slack(torch, g["a_bits"], 0),
               "a2b": slack(torch, g["a_a2b"], PAD), "data": slack(torch, g["a_data"], 0)}
        for K in KS:
            assert n_cols * K < 2 ** 32 and K % 32 == 0 and 64 <= K <= 128
            B0 = rng.uniform(-1, 1, (n_cols, 16)).astype(np.float32)
            B = torch.from_numpy(np.ascontiguousarray(np.tile(B0, (1, K // 16)))).cuda()
            Cd = torch.zeros((c_rows + 8, K), device="cuda")
            p = lambda t: C.c_uint64(t.data_ptr())  # noqa: E731
            args = [p(dev["go"]), p(dev["tco"]), p(dev["ri"]), p(dev["bits"]), p(dev["a2b"]),
                    p(dev["data"]), p(B), p(Cd), C.c_uint32(n_cols - 1), C.c_uint32(K)]
            params = (C.c_void_p * len(args))(*[C.cast(C.byref(a), C.c_void_p) for a in args])
            torch.cuda.synchronize()
            check(cu.cuLaunchKernel(fn, G, 1, 1, 32, K // 32, 1, 0, None, params, None), "cuLaunchKernel")
            check(cu.cuCtxSynchronize(), "cuCtxSynchronize")
            out = Cd[:c_rows].cpu().numpy()
            path = os.path.join(out_dir, f"{case}_adp_k{K}.npz")
            np.savez_compressed(path, B0=B0, C=out, K=np.array([K], np.int32))
            print(f"{case} adaptive K={K}: C {out.shape}, finite {np.isfinite(out).all()} -> {path}")
    return 0


if __name__ == "__main__":
    d = sys.argv[sys.argv.index("--out") + 1] if "--out" in sys.argv else os.path.join(HERE, "ref_spmm")
    if "--adaptive" in sys.argv:
        os.makedirs(d, exist_ok=True)
        sys.exit(main_adaptive(d))
    sys.exit(main())
