"""The allocation-free zlib entry point, r2p_zlib_compress_noalloc.

It serves callers that cannot allocate device memory once running (code
hosted in a framework that owns all GPU memory, latency-bound callers that
must not stall on cudaMalloc/cudaFree): its scratch is a static device array,
so it takes at most 1 MiB of input per call.  Its output must equal the
allocating entry point's (r2p_zlib_compress_device) byte for byte -- the
same exactness every other DEFLATE test here demands -- on consecutive calls
that reuse the shared static scratch.  This file is collected last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def noalloc(r2p, data, level, block_size=0):
    L = r2p.lib()
    n = data.size
    cap = r2p.zlib_bound(n, level, block_size)
    src = r2p.DeviceBuffer.from_array(data)
    dst = r2p.DeviceBuffer(cap)
    ln = r2p.DeviceBuffer(8)
    r2p.check(L.r2p_zlib_compress_noalloc(src.ptr, n, level, block_size, dst.ptr, cap, ln.ptr, None))
    r2p.check(L.r2p_stream_synchronize(None))
    m = int(ln.download(8).view(np.uint64)[0])
    return dst.download(m).tobytes()


def test_noalloc_matches_allocating_entry_point(r2p, engine):
    rng = np.random.default_rng(77)
    cases = [
        (np.repeat(rng.integers(0, 20, size=60000, dtype=np.uint8), 5), 1, 0),                 # 300000 bytes
        ((np.arange(1 << 20) // 13 % 251).astype(np.uint8) ^ rng.integers(0, 3, size=1 << 20, dtype=np.uint8),
         1, 0),                                                                                  # 1 MiB, the limit
        (rng.integers(0, 256, size=200001, dtype=np.uint8), 0, 0),
        (np.tile(np.arange(37, dtype=np.uint8), 5000), 6, 4096),
    ]
    for data, level, bs in cases:
        # two calls in a row: the second reuses the static scratch the first left behind
        for _ in range(2):
            got = noalloc(r2p, data, level, bs)
            want = engine.zlib_compress(data, level, block_size=bs)
            assert got == want
            assert zlib.decompress(got) == data.tobytes()


def test_noalloc_rejects_oversize(r2p):
    L = r2p.lib()
    n = (1 << 20) + 1
    src = r2p.DeviceBuffer(n)
    cap = r2p.zlib_bound(n, 1, 0)
    dst = r2p.DeviceBuffer(cap)
    ln = r2p.DeviceBuffer(8)
    st = L.r2p_zlib_compress_noalloc(src.ptr, n, 1, 0, dst.ptr, cap, ln.ptr, None)
    assert st == r2p.EINVAL
    assert b"1 MiB" in L.r2p_last_error()
