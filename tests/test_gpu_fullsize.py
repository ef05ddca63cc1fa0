"""The benchmark images at their full sizes, through the C ABI.

Size-independent properties only: every chunk CRC, the zlib header and the
Adler-32 trailer check out, the IDAT stream inflates with stock zlib to
exactly the oracle's filtered scanlines, and the unfiltered pixels equal the
oracle's windowed pixels (decode_and_check).  The 3072x3072 16-bit image runs
at level 1 (the autotuned 21760-byte blocks of the built-in table, three LZ77
CTAs per SM) and level 6, and in 65520-byte blocks (one 1024-thread CTA per
block); the 6000x4000 RGB16 image, whose blocks all fall back to stored
blocks, at level 1.
"""
import numpy as np
import pytest

from test_gpu_png import decode_and_check

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("level,block_size", [(1, 0), (1, 65520), (6, 0)])
def test_c1_full_size(engine, O, r2p, W, level, block_size):
    raw = W.radial_rects(1, 3072, 3072)
    img = W.image_c1(level=level)
    img.block_size = block_size
    png = engine.encode_png(img, raw)
    assert len(png) <= r2p.png_bound(img)
    _, stream = decode_and_check(O, r2p, img, raw, png)
    # level 1 stays near 0.67 of the filtered bytes, level 6 near zlib -6's 0.375
    assert len(stream) < (0.70 if level == 1 else 0.40) * img.filtered_bytes


def test_c2_full_size(engine, O, r2p, W):
    raw = W.rgb_sinusoids(2, 6000, 4000)
    img = W.image_c2(level=1)
    png = engine.encode_png(img, raw)
    assert len(png) <= r2p.png_bound(img)
    decode_and_check(O, r2p, img, raw, png)


def test_c1_full_size_many_equals_single(engine, r2p, W):
    """The host-buffer entry point the end-to-end benchmark times gives the
    same bytes as the single call, over more images than it keeps in flight."""
    base = W.radial_rects(1, 3072, 3072)
    raws = [np.ascontiguousarray(np.roll(base, 97 * k, axis=1)) for k in range(2 * r2p.MANY_SLOTS + 1)]
    img = W.image_c1(level=1)
    sts, pngs = engine.encode_png_many([img] * len(raws), raws)
    assert all(s == r2p.OK for s in sts)
    for raw, png in zip(raws, pngs):
        assert png == engine.encode_png(img, raw)
