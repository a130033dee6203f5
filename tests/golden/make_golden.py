"""Generate the golden fixtures in this folder from the reference's own code.

Writes small Matrix Market inputs to ./inputs/, runs the reference's host
format code on each (oracle/_ref/ref_golden, compiled from the AccSpMM
sources by `make -C oracle ref`), and stores what it produced as ./<name>.npz:
COO, CSR, METCF (rowWindowOffset, tcOffset, tcLocalBit, sparseA2B, data),
AdpBME for the reference driver's parameters (3, 1, 2, 16; src/mma_tf32.cu:222) and for (2, 3, 5, 4), and the
balanceStrategy flag.  Run it where the reference sources exist:

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from accspmm_gb300 import synth  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "ref_golden")
DTYPES = {1: np.uint32, 2: np.uint64, 3: np.float32, 4: np.int32}


def parse_dump(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    pos = 0
    while pos < len(buf):
        name = buf[pos:pos + 16].split(b"\0", 1)[0].decode()
        dtype, count = struct.unpack_from("<IQ", buf, pos + 16)
        pos += 28
        dt = np.dtype(DTYPES[dtype])
        out[name] = np.frombuffer(buf, dtype=dt, count=count, offset=pos).copy()
        pos += count * dt.itemsize
    return out


def hand_written() -> dict:
    """Edge cases written out as Matrix Market text."""
    cases = {}
    # The 10x10 symmetric known-answer case: W=2, T=2.
    cases["kat10"] = (
        "%%MatrixMarket matrix coordinate real symmetric\n"
        "10 10 6\n1 1 1\n3 1 2\n9 2 3\n10 4 4\n5 5 5\n10 9 6\n")
    # Rectangular, rows not a multiple of 8, an empty window (rows 9-16),
    # unsorted columns within rows, a duplicated entry, a comment line.
    cases["ragged_unsorted"] = (
        "%%MatrixMarket matrix coordinate real general\n"
        "% a comment line\n"
        "21 30 14\n"
        "1 5 0.5\n1 2 -1.25\n3 30 2\n2 2 1e-3\n8 1 7\n1 5 0.25\n"
        "17 9 3\n21 21 4\n18 1 -2\n20 30 6\n17 2 8\n19 12 9\n21 1 1\n8 8 0.125\n")
    cases["pattern_sym"] = (
        "%%MatrixMarket matrix coordinate pattern symmetric\n"
        "12 12 7\n1 1\n2 1\n7 3\n9 4\n12 12\n11 2\n10 9\n")
    # complex, 'Hermitian' spelled as the reference expects: real part kept,
    # mirrored without conjugation
    cases["complex_herm"] = (
        "%%MatrixMarket matrix coordinate complex Hermitian\n"
        "9 9 4\n1 1 2 0\n5 2 1.5 -3\n9 1 -4 1\n8 8 1 0\n")
    cases["skew"] = (
        "%%MatrixMarket matrix coordinate real skew-symmetric\n"
        "8 8 3\n2 1 1\n5 3 -2\n8 7 3\n")
    # lower-case 'hermitian' is rejected by the reference's case-sensitive
    # banner check
    cases["herm_lower"] = (
        "%%MatrixMarket matrix coordinate complex hermitian\n"
        "2 2 1\n1 1 1 0\n")
    cases["bad_banner"] = "%MatrixMarket matrix coordinate real general\n2 2 0\n"
    cases["no_size"] = "%%MatrixMarket matrix coordinate real general\n% only comments\n"
    # blank line before the size line is accepted (fscanf fallback)
    cases["blank_size"] = (
        "%%MatrixMarket matrix coordinate real general\n\n3 3 2\n1 1 1\n3 2 2\n")
    return cases


def random_cases() -> dict:
    """Seeded random matrices written by the synthetic generators."""
    cases = {}
    r, c, v = synth.powerlaw_symmetric(n=1000, mean=8.0, d_max=200, seed=3)
    cases["plsym1000"] = (1000, 1000, r, c, v, True)
    # one very long window (rows 0-7 dense-ish) forces AdpBME splits and the
    # adaptive balance decision
    rng = np.random.default_rng(7)
    rows, cols = [], []
    for i in range(64):
        d = 300 if i < 8 else int(rng.integers(1, 6))
        cs = np.unique(rng.integers(0, 600, size=d))
        rows.extend([i] * len(cs))
        cols.extend(cs.tolist())
    rows = np.array(rows, dtype=np.uint32)
    cols = np.array(cols, dtype=np.uint32)
    vals = rng.random(len(rows), dtype=np.float32)
    cases["longwin"] = (64, 600, rows, cols, vals, False)
    rng = np.random.default_rng(11)
    nr, nc = 203, 157
    dens = rng.random((nr, nc)) < 0.05
    rr, cc = np.nonzero(dens)
    vv = rng.uniform(-1, 1, size=rr.size).astype(np.float32)
    cases["rand203"] = (nr, nc, rr.astype(np.uint32), cc.astype(np.uint32), vv, False)
    return cases


def main() -> None:
    if not os.path.exists(REF_BIN):
        raise SystemExit(f"missing {REF_BIN}: run `make -C oracle ref` first")
    inp = os.path.join(HERE, "inputs")
    os.makedirs(inp, exist_ok=True)
    paths = {}
    for name, text in hand_written().items():
        p = os.path.join(inp, name + ".mtx")
        with open(p, "w") as f:
            f.write(text)
        paths[name] = p
    for name, (nr, nc, r, c, v, sym) in random_cases().items():
        p = os.path.join(inp, name + ".mtx")
        synth.write_mtx(p, nr, nc, r, c, v, symmetric=sym)
        paths[name] = p
    for name, p in sorted(paths.items()):
        tmp = os.path.join(HERE, name + ".bin")
        subprocess.run([REF_BIN, p, tmp], check=True, stdout=subprocess.DEVNULL)
        d = parse_dump(tmp)
        os.remove(tmp)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        st = int(d["status"][0])
        extra = ""
        if st == 0:
            extra = f" dims={d['dims'].tolist()} tiles={len(d['m_bits'])}"
            if "balance" in d:
                extra += f" adaptive={int(d['balance'][0])}"
        print(f"{name}: status={st}{extra}")


if __name__ == "__main__":
    main()
