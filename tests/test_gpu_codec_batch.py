"""Many queues per codec call: every stream of a batch equals the reference's
stream for that queue, and decoding the batch gives every queue back."""
import os

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

g5 = pytest.importorskip("gpugraph500_gb300")
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def codec():
    c = g5.Codec(1 << 22)
    yield c
    c.close()


def to_dev(a, extra=4):
    a = np.ascontiguousarray(a, dtype=np.uint32)
    t = torch.zeros(len(a) + extra, dtype=torch.int32, device="cuda")
    if len(a):
        t[:len(a)] = torch.from_numpy(a.view(np.int32)).cuda()
    return t


def u32(t):
    return t.cpu().numpy().view(np.uint32)


def batch_round_trip(codec, queues, mode, thr=0):
    in_off = np.zeros(len(queues) + 1, np.uint64)
    in_off[1:] = np.cumsum([len(q) for q in queues])
    din = to_dev(np.concatenate(queues) if queues else np.zeros(0, np.uint32))
    dout = torch.zeros(g5.Codec.batch_bound(in_off) + 4, dtype=torch.int32, device="cuda")
    out_off, words = codec.encode_batch(din, in_off, dout, raw_threshold=thr, mode=mode)
    host = u32(dout)
    streams = [host[int(o):int(o) + int(w)] for o, w in zip(out_off[:-1], words)]
    back = torch.zeros(int(in_off[-1]) + 4, dtype=torch.int32, device="cuda")
    n = np.diff(in_off)
    boff, ok = codec.decode_batch(dout, out_off[:-1], words, n, back, raw_threshold=thr, mode=mode)
    assert ok.all()
    assert np.array_equal(boff, in_off)
    b = u32(back)
    for q, x in enumerate(queues):
        assert np.array_equal(b[int(boff[q]):int(boff[q + 1])], x), q
    return streams


@pytest.mark.parametrize("key,mode", [("d4", g5.CODEC_D4), ("dm", g5.CODEC_DM)])
def test_reference_streams_in_one_batch(codec, golden_dir, key, mode):
    fx = np.load(os.path.join(golden_dir, "codec.npz"))
    ins, io, st, so = fx["inputs"], fx["in_off"], fx[key], fx[key + "_off"]
    queues = [ins[io[i]:io[i + 1]].astype(np.uint32) for i in range(len(io) - 1)]
    streams = batch_round_trip(codec, queues, mode)
    for i, s in enumerate(streams):
        assert np.array_equal(s, st[so[i]:so[i + 1]]), (fx["kinds"][i], len(queues[i]))


def test_plugin_semantics_in_one_batch(codec, golden_dir):
    fx = np.load(os.path.join(golden_dir, "codec.npz"))
    pin, po, out, oo = fx["plugin_in"], fx["plugin_in_off"], fx["plugin_out"], fx["plugin_out_off"]
    queues = [pin[po[i]:po[i + 1]].astype(np.uint32) for i in range(len(po) - 1)]
    streams = batch_round_trip(codec, queues, g5.CODEC_DM, thr=64)
    for i, s in enumerate(streams):
        assert np.array_equal(s, out[oo[i]:oo[i + 1]]), len(queues[i])


def test_level_queues_in_one_batch(codec, golden_dir):
    fx = np.load(os.path.join(golden_dir, "levels_s12.npz"))
    qo, so = fx["q_off"], fx["s_off"]
    queues = [fx["queues"][qo[L - 1]:qo[L]].astype(np.uint32) for L in range(1, len(qo))]
    streams = batch_round_trip(codec, queues, g5.CODEC_D4)
    for L, s in enumerate(streams):
        assert np.array_equal(s, fx["streams"][so[L]:so[L + 1]])


@pytest.mark.parametrize("mode,omode", [(g5.CODEC_D4, orc.D4), (g5.CODEC_DM, orc.DM)])
def test_random_mix_matches_oracle(codec, mode, omode):
    rng = np.random.default_rng(23)
    sizes = [0, 1, 5, 127, 128, 129, 255, 2048, 2049, 16 * 128 * 3 + 17, 0, 70000, 3, 300001, 64, 65]
    queues = [np.sort(rng.choice(1 << 27, size=n, replace=False)).astype(np.uint32) for n in sizes]
    streams = batch_round_trip(codec, queues, mode)
    for q, s in zip(queues, streams):
        assert np.array_equal(s, orc.encode(q, omode)), len(q)
    # the same queues again on the same workspace (it keeps no state between calls)
    streams2 = batch_round_trip(codec, queues[::-1], mode)
    for q, s in zip(queues[::-1], streams2):
        assert np.array_equal(s, orc.encode(q, omode)), len(q)


def test_one_corrupt_stream_is_flagged(codec):
    rng = np.random.default_rng(3)
    queues = [np.sort(rng.choice(1 << 24, size=n, replace=False)).astype(np.uint32) for n in (5000, 40000, 9000)]
    in_off = np.zeros(4, np.uint64)
    in_off[1:] = np.cumsum([len(q) for q in queues])
    din = to_dev(np.concatenate(queues))
    dout = torch.zeros(g5.Codec.batch_bound(in_off) + 4, dtype=torch.int32, device="cuda")
    out_off, words = codec.encode_batch(din, in_off, dout)
    bad = dout.clone()
    bad[int(out_off[1]) + 1] = 0  # a cookie of stream 1
    back = torch.zeros(int(in_off[-1]) + 512, dtype=torch.int32, device="cuda")
    with pytest.raises(g5.G5Error) as e:
        codec.decode_batch(bad, out_off[:-1], words, np.diff(in_off), back)
    assert e.value.stream_ok.tolist() == [1, 0, 1]
    b = u32(back)
    for q in (0, 2):  # the well-formed streams still decode
        assert np.array_equal(b[int(in_off[q]):int(in_off[q + 1])], queues[q])
    # a stream that claims more values than it holds
    n = np.diff(in_off).copy()
    n[2] += 128
    with pytest.raises(g5.G5Error) as e:
        codec.decode_batch(dout, out_off[:-1], words, n, back)
    assert e.value.stream_ok.tolist() == [1, 1, 0]
