"""Generates the golden fixtures in tests/golden from the reference itself.

Runs only where the read-only gpugraph500 tree is present: it builds
oracle/_ref/libg5ref.so (the reference's own generator, CSR build, CPU BFS,
validator and SIMD codec, compiled from their sources by oracle/Makefile)
and records its outputs:

  codec.npz     s4-bp128-d4 / -dm streams of the reference codec library for
                many input shapes, and the reference CpuSimd plugin's streams
  kron_s10.npz  scale-10 Kronecker edge list, CSR, roots, parents of 16 roots,
                TEPS edge counts and validator verdicts of 64 roots
  kron_s16.json scale-16 digests: edge-list / CSR sha256, 64 roots, per-root
                parent sha256, TEPS edge counts, depths
  levels_s12.npz per-level sorted frontier queues of one scale-12 search and
                their reference d4 streams

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "libg5ref.so")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load_ref():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    r = C.CDLL(REF)
    SZ, I64 = C.c_size_t, C.c_int64
    for f in ("ref_codec_encode", "ref_codec_decode", "ref_plugin_compress", "ref_plugin_decompress"):
        getattr(r, f).restype = SZ
    r.ref_make_graph.restype = I64
    r.ref_setup.restype = I64
    r.ref_nnz.restype = I64
    return r


P = lambda a: a.ctypes.data_as(C.c_void_p)


def ref_graph(r, scale):
    m = 16 << scale
    e = np.zeros((m, 2), np.int64)
    r.ref_make_graph(scale, 16, C.c_uint64(1), C.c_uint64(2), P(e))
    n = r.ref_setup(P(e), C.c_int64(m))
    nnz = r.ref_nnz()
    ro = np.zeros(n + 1, np.int64)
    col = np.zeros(nnz, np.int64)
    r.ref_csr(P(ro), P(col))
    roots = np.zeros(64, np.int64)
    k = r.ref_roots(64, P(roots))
    return e, n, ro, col.astype(np.uint32), roots[:k]


def ref_bfs(r, n, root):
    pred = np.zeros(n, np.int64)
    valid, ne = C.c_int(), C.c_int64()
    depth = r.ref_bfs(C.c_int64(int(root)), P(pred), C.byref(valid), C.byref(ne))
    return pred, valid.value, ne.value, depth


def codec_inputs():
    rng = np.random.default_rng(20261203)
    cases = []
    for n in [0, 1, 5, 64, 65, 127, 128, 129, 255, 256, 1000, 2047, 2048, 2049, 2176, 4096, 5000]:
        cases.append(("sorted", np.sort(rng.choice(1 << 24, size=n, replace=False)).astype(np.uint32)))
        cases.append(("random", rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)))
        cases.append(("wide", np.sort(rng.integers(0, 1 << 32, size=n, dtype=np.uint64)).astype(np.uint32)))
        cases.append(("const", np.full(n, 7, np.uint32)))
    # every bit width 0..32 in one miniblock each: deltas of exactly b bits
    for b in range(33):
        x = np.zeros(128 * 3, np.uint64)
        d = (1 << b) - 1 if b else 0
        x = np.cumsum(np.full(128 * 3, d, np.uint64)) & 0xFFFFFFFF
        cases.append((f"bits{b}", x.astype(np.uint32)))
    return cases


def main() -> int:
    if not os.path.isdir("/root/reference"):
        print("reference tree not present; fixtures unchanged")
        return 0
    r = load_ref()
    # ---- codec ----
    cases = codec_inputs()
    ins, offs, kinds = [], [0], []
    streams = {"d4": ([], [0]), "dm": ([], [0])}
    for kind, x in cases:
        ins.append(x)
        offs.append(offs[-1] + len(x))
        kinds.append(kind)
        for name in ("d4", "dm"):
            cap = len(x) * 2 + 64
            o = np.zeros(cap, np.uint32)
            w = r.ref_codec_encode(f"s4-bp128-{name}".encode(), P(x), len(x), P(o), cap)
            streams[name][0].append(o[:w].copy())
            streams[name][1].append(streams[name][1][-1] + w)
    # plugin streams: CpuSimd reconfigured to "s4-bp128-d4", threshold 64
    rng = np.random.default_rng(7)
    pin, poff, pout, pwoff = [], [0], [], [0]
    for n in [1, 10, 64, 65, 128, 300, 1000, 4100]:
        x = np.sort(rng.choice(1 << 22, size=n, replace=False)).astype(np.int64)
        o = np.zeros(n + 64, np.uint32)
        w = r.ref_plugin_compress(64, b"s4-bp128-d4", P(x), n, P(o))
        pin.append(x)
        poff.append(poff[-1] + n)
        pout.append(o[:w].copy())
        pwoff.append(pwoff[-1] + w)
    np.savez_compressed(
        os.path.join(HERE, "codec.npz"),
        inputs=np.concatenate(ins), in_off=np.array(offs, np.int64), kinds=np.array(kinds),
        d4=np.concatenate(streams["d4"][0]), d4_off=np.array(streams["d4"][1], np.int64),
        dm=np.concatenate(streams["dm"][0]), dm_off=np.array(streams["dm"][1], np.int64),
        plugin_in=np.concatenate(pin), plugin_in_off=np.array(poff, np.int64),
        plugin_out=np.concatenate(pout), plugin_out_off=np.array(pwoff, np.int64),
    )
    # ---- scale 10 ----
    e, n, ro, col, roots = ref_graph(r, 10)
    preds, valid, nedge, depth = [], [], [], []
    for i, root in enumerate(roots):
        p, v, ne, d = ref_bfs(r, n, root)
        valid.append(v)
        nedge.append(ne)
        depth.append(d)
        if i < 16:
            preds.append(p)
    np.savez_compressed(os.path.join(HERE, "kron_s10.npz"), edges=e, n=n, row_off=ro, col=col, roots=roots,
                        preds=np.stack(preds), valid=np.array(valid), nedge=np.array(nedge),
                        depth=np.array(depth))
    # ---- scale 16 digests ----
    e, n, ro, col, roots = ref_graph(r, 16)
    info = {"scale": 16, "edgefactor": 16, "seed": [1, 2], "n": int(n), "nnz": int(len(col)),
            "edges_sha256": sha(e), "row_off_sha256": sha(ro), "col_u32_sha256": sha(col),
            "roots": [int(x) for x in roots], "pred_sha256": [], "nedge": [], "valid": [], "depth": []}
    for root in roots:
        p, v, ne, d = ref_bfs(r, n, root)
        info["pred_sha256"].append(sha(p))
        info["nedge"].append(int(ne))
        info["valid"].append(int(v))
        info["depth"].append(int(d))
    with open(os.path.join(HERE, "kron_s16.json"), "w") as f:
        json.dump(info, f, indent=1)
    # ---- per-level queues of one scale-12 search, reference d4 streams ----
    e, n, ro, col, roots = ref_graph(r, 12)
    p, v, ne, d = ref_bfs(r, n, roots[0])
    # levels from the parent tree
    lev = np.full(n, -1, np.int64)
    lev[roots[0]] = 0
    changed = True
    while changed:
        changed = False
        m = (p >= 0) & (lev < 0)
        idx = np.nonzero(m)[0]
        ok = lev[p[idx]] >= 0
        if ok.any():
            lev[idx[ok]] = lev[p[idx[ok]]] + 1
            changed = True
    qs, qoff, ss, soff = [], [0], [], [0]
    for L in range(1, int(lev.max()) + 1):
        q = np.nonzero(lev == L)[0].astype(np.uint32)
        o = np.zeros(2 * len(q) + 64, np.uint32)
        w = r.ref_codec_encode(b"s4-bp128-d4", P(q), len(q), P(o), len(o))
        qs.append(q)
        qoff.append(qoff[-1] + len(q))
        ss.append(o[:w].copy())
        soff.append(soff[-1] + w)
    np.savez_compressed(os.path.join(HERE, "levels_s12.npz"), root=roots[0], queues=np.concatenate(qs),
                        q_off=np.array(qoff, np.int64), streams=np.concatenate(ss),
                        s_off=np.array(soff, np.int64))
    r.ref_free()
    print("fixtures written to", HERE)
    return 0


if __name__ == "__main__":
    sys.exit(main())
