"""The CPU oracle against golden vectors produced by the reference itself.

The fixtures in tests/golden come from the gpugraph500 sources compiled
unmodified into oracle/_ref (tests/golden/make_golden.py).  These tests pin
the oracle restatement to them; the GPU tests then use the oracle as the
checker at sizes the fixtures do not cover.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as orc


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def codec_fx(golden_dir):
    return np.load(os.path.join(golden_dir, "codec.npz"))


def _cases(fx, key):
    ins, io = fx["inputs"], fx["in_off"]
    st, so = fx[key], fx[key + "_off"]
    for i in range(len(io) - 1):
        yield fx["kinds"][i], ins[io[i]:io[i + 1]], st[so[i]:so[i + 1]]


@pytest.mark.parametrize("key,mode", [("d4", orc.D4), ("dm", orc.DM)])
def test_codec_streams_match_reference(codec_fx, key, mode):
    n = 0
    for kind, x, stream in _cases(codec_fx, key):
        got = orc.encode(x, mode)
        assert np.array_equal(got, stream), (kind, len(x))
        back = orc.decode(stream, len(x) + 8, mode)
        assert back is not None and np.array_equal(back, x), (kind, len(x))
        n += 1
    assert n > 100


def test_plugin_emits_dm_whatever_it_is_told(codec_fx):
    """The reference CpuSimd plugin reconfigured to s4-bp128-d4 still emits dm streams."""
    pin, po = codec_fx["plugin_in"], codec_fx["plugin_in_off"]
    out, oo = codec_fx["plugin_out"], codec_fx["plugin_out_off"]
    for i in range(len(po) - 1):
        x = pin[po[i]:po[i + 1]]
        ref = out[oo[i]:oo[i + 1]]
        assert np.array_equal(orc.plugin_compress(x, 64, orc.DM), ref), len(x)
        if len(x) >= 256:  # d4 and dm differ once there are miniblocks
            assert not np.array_equal(orc.plugin_compress(x, 64, orc.D4), ref)


def test_corrupt_stream_rejected():
    x = np.arange(0, 3000, 3, dtype=np.uint32)
    s = orc.encode(x, orc.D4)
    bad = s.copy()
    bad[1] = 0
    assert orc.decode(bad, 2000, orc.D4) is None
    bad = s.copy()
    bad[4] = 0xFFFFFFFF  # bit widths > 32
    assert orc.decode(bad, 2000, orc.D4) is None


@pytest.fixture(scope="module")
def s10(golden_dir):
    return np.load(os.path.join(golden_dir, "kron_s10.npz"))


def test_generator_csr_roots_s10(s10):
    e = orc.kronecker(10)
    assert np.array_equal(e, s10["edges"])
    n = int(s10["n"])
    ro, col = orc.build_csr(n, e)
    assert np.array_equal(ro, s10["row_off"])
    assert np.array_equal(col, s10["col"])
    assert np.array_equal(orc.select_roots(ro, 64), s10["roots"])


def test_bfs_and_validator_s10(s10):
    n = int(s10["n"])
    ro, col, e = s10["row_off"], s10["col"], s10["edges"]
    for i, root in enumerate(s10["roots"]):
        pred, level = orc.bfs(ro, col, int(root))
        if i < len(s10["preds"]):
            assert np.array_equal(pred, s10["preds"][i])
        ok, ne, depth = orc.validate(n, e, int(root), pred)
        assert ok == bool(s10["valid"][i])
        assert ne == int(s10["nedge"][i])
        assert int(level.max()) + 1 == int(s10["depth"][i])
        assert np.array_equal(depth, level)


def test_kron_s16_digests(golden_dir):
    info = json.load(open(os.path.join(golden_dir, "kron_s16.json")))
    e = orc.kronecker(16)
    assert sha(e) == info["edges_sha256"]
    ro, col = orc.build_csr(info["n"], e)
    assert sha(ro) == info["row_off_sha256"] and sha(col) == info["col_u32_sha256"]
    roots = orc.select_roots(ro, 64)
    assert [int(r) for r in roots] == info["roots"]
    for i, root in enumerate(roots[:16]):
        pred, level = orc.bfs(ro, col, int(root))
        assert sha(pred) == info["pred_sha256"][i]
        ok, ne, _ = orc.validate(info["n"], e, int(root), pred)
        assert ok and ne == info["nedge"][i]


def test_level_queue_streams(golden_dir):
    fx = np.load(os.path.join(golden_dir, "levels_s12.npz"))
    e = orc.kronecker(12)
    ro, col = orc.build_csr(1 << 12, e)
    pred, level = orc.bfs(ro, col, int(fx["root"]))
    qo, so = fx["q_off"], fx["s_off"]
    for L in range(1, len(qo)):
        q = np.nonzero(level == L)[0].astype(np.uint32)
        assert np.array_equal(q, fx["queues"][qo[L - 1]:qo[L]])
        assert np.array_equal(orc.encode(q, orc.D4), fx["streams"][so[L - 1]:so[L]])


def test_validator_rejects_broken_trees(s10):
    n = int(s10["n"])
    ro, col, e = s10["row_off"], s10["col"], s10["edges"]
    root = int(s10["roots"][0])
    pred, _ = orc.bfs(ro, col, root)
    v = int(np.nonzero((pred >= 0) & (np.arange(n) != root))[0][0])
    bad = pred.copy(); bad[v] = v                      # self parent
    assert not orc.validate(n, e, root, bad)[0]
    bad = pred.copy(); bad[root] = -1                  # root not its own parent
    assert not orc.validate(n, e, root, bad)[0]
    bad = pred.copy(); bad[v] = -1                     # coverage hole
    assert not orc.validate(n, e, root, bad)[0]
    far = int(np.nonzero(pred == -1)[0][0]) if (pred == -1).any() else None
    if far is not None:
        bad = pred.copy(); bad[v] = far                # parent outside the tree
        assert not orc.validate(n, e, root, bad)[0]


def test_bitmap_or_oracle():
    rng = np.random.default_rng(1)
    d = rng.integers(0, 2**63, 1000, dtype=np.uint64)
    s = [rng.integers(0, 2**63, 1000, dtype=np.uint64) for _ in range(8)]
    want = d.copy()
    for x in s:
        want |= x
    assert np.array_equal(orc.bitmap_or(d, s), want)


def test_skip_table_is_powers_of_a():
    # A^(2*256^k) composed from the table equals the byte-(k) entry for 2
    m1 = orc.skip_matrix(0, 1).astype(object).reshape(5, 5)
    m2 = orc.skip_matrix(0, 2).astype(object).reshape(5, 5)
    assert ((m1.dot(m1)) % 0x7FFFFFFF == m2).all()
    b1 = orc.skip_matrix(1, 1).astype(object).reshape(5, 5)
    acc = np.identity(5, dtype=object)
    for _ in range(256):
        acc = acc.dot(m1) % 0x7FFFFFFF
    assert (acc == b1).all()


def test_threaded_generator_and_csr_match_serial(golden_dir):
    """The host-thread generator and counting CSR build give the reference's
    arrays: the scale-16 digests, and element-wise equality with the serial
    paths on an odd edge range and thread count."""
    info = json.load(open(os.path.join(golden_dir, "kron_s16.json")))
    e = orc.kronecker(16, threads=5)
    assert sha(e) == info["edges_sha256"]
    ro, col = orc.build_csr(info["n"], e, threads=3)
    assert sha(ro) == info["row_off_sha256"] and sha(col) == info["col_u32_sha256"]
    part = orc.kronecker(12, start=1000, end=23457, threads=7)
    assert np.array_equal(part, orc.kronecker(12, start=1000, end=23457, threads=1))
    e12 = orc.kronecker(12, threads=1)
    a = orc.build_csr(1 << 12, e12, threads=1)
    b = orc.build_csr(1 << 12, e12, threads=6)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_teps_edges_equal_validator_count(s10):
    """The endpoint-count form of the TEPS edge count equals the validator's
    edge sweep (validate.h:440-443,485) and the reference-run fixture."""
    n = int(s10["n"])
    ro, col, e = s10["row_off"], s10["col"], s10["edges"]
    deg = orc.endpoint_counts(n, e)
    assert int(deg.sum()) == 2 * len(e)
    for i, root in enumerate(s10["roots"][:16]):
        pred, _ = orc.bfs(ro, col, int(root))
        ok, ne, _ = orc.validate(n, e, int(root), pred)
        assert orc.teps_edges(deg, pred) == ne == int(s10["nedge"][i])
