"""The C ABI library: it loads without a GPU, exports every symbol that
include/r2p.h declares, its host-side arithmetic matches zlib, and its
calls fail with a status (never exit) when no GPU is usable."""
import ctypes
import os
import re
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(r2p_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(r2p):
    lib = ctypes.CDLL(r2p.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
        assert n in r2p.SIGNATURES, "binding lacks " + n


def test_host_crc_and_adler_combine(r2p):
    rng = np.random.default_rng(0)
    buf = rng.integers(0, 256, size=200000, dtype=np.uint8).tobytes()
    for n1, n2 in ((0, 5), (5, 0), (1, 1), (1000, 199000), (65536, 65536), (123457, 3)):
        a, b = buf[:n1], buf[n1:n1 + n2]
        assert r2p.crc32_combine(zlib.crc32(a), zlib.crc32(b), n2) == zlib.crc32(a + b)
        assert r2p.adler32_combine(zlib.adler32(a), zlib.adler32(b), n2) == zlib.adler32(a + b)


def test_png_bound_and_validation(r2p, W):
    img = W.image_c0()
    nb = -(-img.filtered_bytes // 1024)
    assert r2p.png_bound(img) == 43 + img.filtered_bytes + 5 * nb + 20
    img.block_size = r2p.BLOCK64
    assert r2p.png_bound(img) == 43 + img.filtered_bytes + 5 * 5 + 20
    bad = W.image_c0()
    bad.channels = 2
    assert r2p.png_bound(bad) == 0
    bad = W.image_c0()
    bad.dicom.high_bit = 9          # shift -2: the reference's table index would be undefined
    assert r2p.png_bound(bad) == 0
    assert r2p.zlib_bound(100, 0) == 2 + 100 + 5 * 2 + 4


def test_no_gpu_reports_status(r2p):
    import torch
    if torch.cuda.is_available():
        return
    p = ctypes.c_void_p()
    st = r2p.lib().r2p_engine_create(0, 0, ctypes.byref(p))
    assert st in (r2p.ECUDA, r2p.EINVAL)
    assert p.value is None
    assert r2p.lib().r2p_last_error()
