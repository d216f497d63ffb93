"""g5_codec_encode_noalloc: the encoder for callers that cannot allocate
device memory (its scratch is a static array in the library).

Named to be collected last.  Calls the C ABI directly and checks, on two calls
in a row, that it writes exactly the stream of the allocating entry point
g5_codec_encode and of the oracle encoder; that a warm call leaves the
device's free memory unchanged (it allocates nothing); and that the size
limit is enforced.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu

g5 = pytest.importorskip("gpugraph500_gb300")
torch = pytest.importorskip("torch")

LIMIT = 1 << 20


def _encode_both(lib, codec, x, mode):
    n = len(x)
    din = torch.zeros(max(n, 4) + 4, dtype=torch.int32, device="cuda")
    if n:
        din[:n] = torch.from_numpy(x.view(np.int32)).cuda()
    cap = lib.g5_codec_bound(n) + 8
    want = torch.zeros(cap, dtype=torch.int32, device="cuda")
    got = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    w1, w2 = C.c_size_t(), C.c_size_t()
    assert lib.g5_codec_encode(codec, din.data_ptr(), n, want.data_ptr(), C.byref(w1), mode, None) == 0
    assert lib.g5_codec_encode_noalloc(din.data_ptr(), n, got.data_ptr(), C.byref(w2), mode, None) == 0
    return w1.value, w2.value, want[:w1.value].cpu().numpy(), got[:w2.value].cpu().numpy()


@pytest.mark.parametrize("mode", [g5.CODEC_D4, g5.CODEC_DM])
def test_noalloc_matches_allocating_encoder_twice(mode):
    lib = g5.lib()
    h = C.c_void_p()
    assert lib.g5_codec_create(LIMIT, C.byref(h)) == 0
    rng = np.random.default_rng(123)
    # two calls in a row: a large queue, then a smaller one (stale scratch
    # from the first call must not leak into the second)
    for n in (LIMIT - 77, 5000):
        x = np.sort(rng.choice(1 << 26, size=n, replace=False)).astype(np.uint32)
        w1, w2, want, got = _encode_both(lib, h, x, mode)
        assert w1 == w2
        assert np.array_equal(want, got)
        ref = orc.encode(x, orc.D4 if mode == g5.CODEC_D4 else orc.DM)
        assert np.array_equal(got.view(np.uint32), ref)
    lib.g5_codec_destroy(h)


def test_noalloc_warm_call_allocates_nothing():
    """After a first (set-up) call, a call leaves the device's free memory
    exactly as it was."""
    lib = g5.lib()
    n = 200_000
    x = np.arange(0, 3 * n, 3, dtype=np.uint32)
    din = torch.from_numpy(x.view(np.int32)).cuda()
    dout = torch.zeros(lib.g5_codec_bound(n) + 8, dtype=torch.int32, device="cuda")
    w = C.c_size_t()
    assert lib.g5_codec_encode_noalloc(din.data_ptr(), n, dout.data_ptr(), C.byref(w), g5.CODEC_D4, None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert lib.g5_codec_encode_noalloc(din.data_ptr(), n, dout.data_ptr(), C.byref(w), g5.CODEC_D4, None) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(dout[:w.value].cpu().numpy().view(np.uint32), orc.encode(x, orc.D4))


def test_noalloc_rejects_oversize_and_bad_args():
    lib = g5.lib()
    din = torch.zeros(16, dtype=torch.int32, device="cuda")
    dout = torch.zeros(16, dtype=torch.int32, device="cuda")
    w = C.c_size_t()
    assert lib.g5_codec_encode_noalloc(din.data_ptr(), LIMIT + 1, dout.data_ptr(), C.byref(w),
                                       g5.CODEC_D4, None) == g5.G5_ERR_CAPACITY
    assert lib.g5_codec_encode_noalloc(din.data_ptr(), 8, dout.data_ptr(), C.byref(w), 9, None) == \
        g5.G5_ERR_INVALID_ARG
