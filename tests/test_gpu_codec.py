"""The device codec against the reference streams and the oracle."""
import os

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

g5 = pytest.importorskip("gpugraph500_gb300")
torch = pytest.importorskip("torch")


def dev(a):
    t = torch.from_numpy(np.ascontiguousarray(a).view(np.int32) if a.dtype == np.uint32 else a).cuda()
    return t


def host_u32(t, n):
    return t[:n].cpu().numpy().view(np.uint32)


@pytest.fixture(scope="module")
def codec():
    c = g5.Codec(1 << 22)
    yield c
    c.close()


def enc_dec(codec, x, mode):
    n = len(x)
    din = torch.zeros(max(n, 4) + 4, dtype=torch.int32, device="cuda")
    if n:
        din[:n] = torch.from_numpy(x.view(np.int32)).cuda()
    cap = g5.Codec.bound(n) + 8
    dout = torch.zeros(cap, dtype=torch.int32, device="cuda")
    w = codec.encode(din, n, dout, mode)
    stream = host_u32(dout, w)
    back = torch.zeros(max(n, 4) + 132, dtype=torch.int32, device="cuda")
    m = codec.decode(dout, w, back, n + 128, mode)
    return stream, host_u32(back, m)


@pytest.mark.parametrize("key,mode", [("d4", g5.CODEC_D4), ("dm", g5.CODEC_DM)])
def test_reference_streams(codec, golden_dir, key, mode):
    fx = np.load(os.path.join(golden_dir, "codec.npz"))
    ins, io, st, so = fx["inputs"], fx["in_off"], fx[key], fx[key + "_off"]
    for i in range(len(io) - 1):
        x = ins[io[i]:io[i + 1]]
        stream, back = enc_dec(codec, x, mode)
        assert np.array_equal(stream, st[so[i]:so[i + 1]]), (fx["kinds"][i], len(x))
        assert np.array_equal(back, x), (fx["kinds"][i], len(x))


@pytest.mark.parametrize("mode,omode", [(g5.CODEC_D4, orc.D4), (g5.CODEC_DM, orc.DM)])
def test_large_queues_match_oracle(codec, mode, omode):
    rng = np.random.default_rng(11)
    for n in (128 * 16 * 40 + 77, 1 << 20, (1 << 22) - 5):
        x = np.sort(rng.choice(1 << 26, size=n, replace=False)).astype(np.uint32)
        stream, back = enc_dec(codec, x, mode)
        assert np.array_equal(stream, orc.encode(x, omode))
        assert np.array_equal(back, x)


def test_encoder_ranges_longer_than_one_chunk():
    """Over 318 M values every encoder block's range holds more than 512
    groups, so the packing pass places its groups in several chunks."""
    n = 330_000_123
    rng = np.random.default_rng(5)
    x = np.cumsum(rng.integers(1, 16, size=n, dtype=np.uint8), dtype=np.uint32)
    c = g5.Codec(n)
    try:
        din = torch.from_numpy(x.view(np.int32)).cuda()
        dout = torch.empty(g5.Codec.bound(n) + 8, dtype=torch.int32, device="cuda")
        w = c.encode(din, n, dout, g5.CODEC_D4)
        assert np.array_equal(host_u32(dout, w), orc.encode(x, orc.D4))
        del din
        back = torch.empty(n + 132, dtype=torch.int32, device="cuda")
        assert c.decode(dout, w, back, n + 128, g5.CODEC_D4) == n
        assert torch.equal(back[:n].cpu(), torch.from_numpy(x.view(np.int32)))
    finally:
        c.close()


def test_level_queues(codec, golden_dir):
    fx = np.load(os.path.join(golden_dir, "levels_s12.npz"))
    qo, so = fx["q_off"], fx["s_off"]
    for L in range(1, len(qo)):
        q = fx["queues"][qo[L - 1]:qo[L]]
        stream, back = enc_dec(codec, q, g5.CODEC_D4)
        assert np.array_equal(stream, fx["streams"][so[L - 1]:so[L]])
        assert np.array_equal(back, q)


def test_corrupt_streams_are_rejected(codec):
    x = np.arange(0, 30000, 3, dtype=np.uint32)
    s = orc.encode(x, orc.D4)
    cases = []
    b = s.copy(); b[1] = 0; cases.append(b)                  # cookie
    b = s.copy(); b[0] = 127; cases.append(b)                 # n1 not a multiple of 128
    b = s.copy(); b[4] = 0x21212121; cases.append(b)          # widths > 32
    b = s.copy(); b[0] = 1 << 30; cases.append(b)             # longer than capacity
    cases.append(s[:len(s) // 2].copy())                      # truncated
    for bad in cases:
        din = torch.from_numpy(bad.view(np.int32)).cuda()
        out = torch.zeros(len(x) + 256, dtype=torch.int32, device="cuda")
        with pytest.raises(g5.G5Error):
            codec.decode(din, len(bad), out, len(x) + 128, g5.CODEC_D4)


def test_plugin_matches_reference_plugin(golden_dir):
    fx = np.load(os.path.join(golden_dir, "codec.npz"))
    pin, po, out, oo = fx["plugin_in"], fx["plugin_in_off"], fx["plugin_out"], fx["plugin_out_off"]
    p = g5.GpuSimd()
    p.reconfigure(64, "s4-bp128-dm")
    for i in range(len(po) - 1):
        x = pin[po[i]:po[i + 1]]
        c, cs = p.compress(x)
        assert np.array_equal(c, out[oo[i]:oo[i + 1]])
        assert p.isCompressed(len(x), cs) == (len(x) > 64 and cs != len(x))
        back = p.decompress(c, cs, len(x))
        assert np.array_equal(back, x)


def test_bitmap_or_matches_oracle():
    rng = np.random.default_rng(5)
    for words, k in ((1, 1), (7, 3), (1 << 18, 8), (1 << 19 | 1, 5)):
        d = rng.integers(0, 2**63, words, dtype=np.uint64)
        s = [rng.integers(0, 2**63, words, dtype=np.uint64) for _ in range(k)]
        want = orc.bitmap_or(d, s)
        dd = torch.from_numpy(d.view(np.int64)).cuda()
        ss = [torch.from_numpy(x.view(np.int64)).cuda() for x in s]
        g5.bitmap_or(dd, ss, words)
        torch.cuda.synchronize()
        assert np.array_equal(dd.cpu().numpy().view(np.uint64), want)
