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
        # dynamic Huffman at the default 65520-byte blocks, a length no block size divides
        ((np.arange(200003) // 7 % 61).astype(np.uint8) ^ rng.integers(0, 2, size=200003, dtype=np.uint8), 9, 0),
    ]
    for data, level, bs in cases:
        # two calls in a row: the second reuses the static scratch the first left behind
        for _ in range(2):
            got = noalloc(r2p, data, level, bs)
            want = engine.zlib_compress(data, level, block_size=bs)
            assert got == want
            assert zlib.decompress(got) == data.tobytes()


def test_noalloc_allocates_nothing(r2p):
    """Once set up, calls leave the device's free memory where it was: no
    cudaMalloc behind the entry point, nor a pool that grows."""
    torch = pytest.importorskip("torch")
    L = r2p.lib()
    data = (np.arange(1 << 20) // 9 % 200).astype(np.uint8)
    src = r2p.DeviceBuffer.from_array(data)
    cap = r2p.zlib_bound(data.size, 1, 0)
    dst = r2p.DeviceBuffer(cap)
    ln = r2p.DeviceBuffer(8)
    for level in (1, 6, 0):   # set-up and first use of every kernel
        r2p.check(L.r2p_zlib_compress_noalloc(src.ptr, data.size, level, 0, dst.ptr, cap, ln.ptr, None))
    r2p.check(L.r2p_stream_synchronize(None))
    free0, _ = torch.cuda.mem_get_info()
    for level in (1, 6, 0, 1):
        r2p.check(L.r2p_zlib_compress_noalloc(src.ptr, data.size, level, 0, dst.ptr, cap, ln.ptr, None))
    r2p.check(L.r2p_stream_synchronize(None))
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_in_a_process_without_an_engine(tmp_path):
    """A fresh process that never creates an engine: the entry point sets
    itself up and compresses on its own."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import sys, zlib\n"
        "import numpy as np\n"
        "sys.path.insert(0, %r)\n"
        "import __graft_entry__ as g\n"
        "r2p = g.load_package()\n"
        "L = r2p.lib()\n"
        "data = (np.arange(300001) // 11 %% 97).astype(np.uint8)\n"
        "src = r2p.DeviceBuffer.from_array(data)\n"
        "cap = r2p.zlib_bound(data.size, 1, 0)\n"
        "dst = r2p.DeviceBuffer(cap)\n"
        "ln = r2p.DeviceBuffer(8)\n"
        "for _ in range(2):\n"
        "    r2p.check(L.r2p_zlib_compress_noalloc(src.ptr, data.size, 1, 0, dst.ptr, cap, ln.ptr, None))\n"
        "    r2p.check(L.r2p_stream_synchronize(None))\n"
        "    m = int(ln.download(8).view(np.uint64)[0])\n"
        "    assert zlib.decompress(dst.download(m).tobytes()) == data.tobytes()\n"
        "print('ok')\n" % root)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr


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
