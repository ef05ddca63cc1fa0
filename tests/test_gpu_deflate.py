"""DEFLATE on the GPU: level 1 is LZ77 + fixed Huffman, levels 2-9 dynamic
Huffman blocks over a run-length parse.

The compressed bytes are not pinned to the reference (its GPU encoder and
zlib emit different but equivalent streams); every stream must inflate with
stock zlib to exactly the input bytes, and PNGs must decode to the oracle's
pixels.  Compression must also be real: sizes are compared with zlib.
"""
import zlib

import numpy as np
import pytest

from test_gpu_png import decode_and_check

pytestmark = pytest.mark.gpu


def patterns():
    rng = np.random.default_rng(0)
    yield "zeros", np.zeros(200000, np.uint8)
    yield "random", rng.integers(0, 256, size=150001, dtype=np.uint8)
    yield "period7", np.tile(np.arange(7, dtype=np.uint8), 30000)
    yield "smallvals", rng.integers(0, 6, size=130000, dtype=np.uint8)
    yield "runs", np.repeat(rng.integers(0, 256, size=4000, dtype=np.uint8), rng.integers(1, 300, size=4000))
    yield "one", np.array([42], np.uint8)
    yield "three", np.array([1, 2, 3], np.uint8)
    txt = (b"the quick brown fox jumps over the lazy dog; " * 3000)[:100003]
    yield "text", np.frombuffer(txt, np.uint8)
    yield "high_literals", (rng.integers(144, 256, size=70000, dtype=np.uint8))


@pytest.mark.parametrize("name,data", list(patterns()))
@pytest.mark.parametrize("level", [1, 6])
def test_inflate_exact(engine, name, data, level):
    z = engine.zlib_compress(data, level)
    assert zlib.decompress(z) == data.tobytes()
    if name in ("zeros", "runs") or (level == 1 and name in ("period7", "text")):
        assert len(z) < 0.2 * data.size, (name, len(z))
    if level >= 2 and name in ("period7", "text", "smallvals"):
        # run-length parse: repeats farther back than one byte are left to the
        # Huffman code, which still beats the 8-9 bits of a fixed literal
        assert len(z) < 0.6 * data.size, (name, len(z))
    if level >= 2 and name == "random":
        assert len(z) <= data.size + 5 * (data.size // 65520 + 1) + 6     # stored blocks


@pytest.mark.parametrize("level", [1, 6])
# 21760 / 21776 and 32768 / 32784 straddle the LZ77 launch's change of CTA size
@pytest.mark.parametrize("bs", [1024, 4096, 21760, 21776, 32752, 32768, 32784, 65520])
def test_block_sizes(engine, bs, level):
    rng = np.random.default_rng(bs)
    data = np.repeat(rng.integers(0, 16, size=30000, dtype=np.uint8), 7)
    z = engine.zlib_compress(data, level, block_size=bs)
    assert zlib.decompress(z) == data.tobytes()


def test_c1_shape_png(engine, O, r2p, W):
    raw = W.radial_rects(1, 640, 480)
    img = r2p.Image.make(640, 480, 1, 2, r2p.WINDOW_DICOM16, r2p.DicomParams.make(16, 12, 11, 0, wc=2048.0,
                                                                                     ww=4096.0), level=1)
    png = engine.encode_png(img, raw)
    ihdr, stream = decode_and_check(O, r2p, img, raw, png)
    filt_size = img.filtered_bytes
    z1 = len(zlib.compress(O.parse_png(png)[4].tobytes(), 1))
    assert len(stream) < filt_size            # real compression
    # within reach of zlib level 1: fixed Huffman codes (8-9 bits per literal)
    # against zlib's dynamic ones cost ~1.65x on filtered 16-bit residuals
    assert len(stream) < 1.75 * z1


@pytest.mark.parametrize("level", [2, 6, 9])
def test_c1_shape_png_dynamic(engine, O, r2p, W, level):
    raw = W.radial_rects(1, 640, 480)
    img = r2p.Image.make(640, 480, 1, 2, r2p.WINDOW_DICOM16, r2p.DicomParams.make(16, 12, 11, 0, wc=2048.0,
                                                                                     ww=4096.0), level=level)
    png = engine.encode_png(img, raw)
    ihdr, stream = decode_and_check(O, r2p, img, raw, png)
    filt = O.parse_png(png)[4].tobytes()
    # dynamic Huffman over runs: within a few percent of zlib level 6 on
    # filtered scanlines (zlib's own run-length strategy does better than -6)
    assert len(stream) < 1.05 * len(zlib.compress(filt, 6))


def test_c2_shape_png(engine, O, r2p, W):
    raw = W.rgb_sinusoids(2, 1200, 300)
    img = r2p.Image.make(1200, 300, 3, 2, r2p.WINDOW_NONE, level=1)
    decode_and_check(O, r2p, img, raw, engine.encode_png(img, raw))


def test_c0_level1_and_batch_mixed_levels(engine, O, r2p, W):
    imgs, raws, bufs, outs, caps = [], [], [], [], []
    for i, (w, h, lvl) in enumerate([(512, 512, 1), (256, 256, 0), (1024, 100, 6), (300, 7, 1)]):
        raw = W.ct_phantom(30 + i, w, h)
        img = W.image_ct8(w, h, 40.0, 400.0 + 100 * i, level=lvl)
        imgs.append(img)
        raws.append(raw)
        bufs.append(r2p.DeviceBuffer.from_array(raw))
        caps.append(r2p.png_bound(img))
        outs.append(r2p.DeviceBuffer(caps[-1]))
    lens = r2p.DeviceBuffer(8 * len(imgs))
    engine.encode_batch_device(imgs, [b.ptr for b in bufs], [o.ptr for o in outs], caps, lens.ptr)
    n = lens.download(8 * len(imgs)).view(np.uint64)
    for i in range(len(imgs)):
        decode_and_check(O, r2p, imgs[i], raws[i], outs[i].download(int(n[i])).tobytes())


def test_deterministic_output(engine, W, r2p):
    raw = W.radial_rects(5, 512, 300)
    img = r2p.Image.make(512, 300, 1, 2, r2p.WINDOW_DICOM16, r2p.DicomParams.make(16, 12, 11, 0, wc=2048.0,
                                                                                     ww=4096.0), level=1)
    a = engine.encode_png(img, raw)
    b = engine.encode_png(img, raw)
    assert a == b


@pytest.mark.parametrize("level", [0, 1, 6])
def test_raw_deflate_parts_concatenate(engine, level):
    """r2p_deflate_raw_device: open parts (no BFINAL, byte-aligned end) and a
    final part concatenate into one raw DEFLATE stream that stock zlib
    inflates to the input, each part reporting its own Adler-32 -- the
    compress_strip contract (include/compression_backend.h:33-43)."""
    rng = np.random.default_rng(77 + level)
    sizes = [70001, 1, 65520, 200000, 4097]
    pieces = []
    for i, n in enumerate(sizes):
        base = rng.integers(0, 6, size=n, dtype=np.uint8)
        base[::7] = rng.integers(0, 256, size=base[::7].size, dtype=np.uint8)
        pieces.append(base)
    stream, total = b"", b""
    for i, p in enumerate(pieces):
        last = i == len(pieces) - 1
        part, adler = engine.deflate_raw(p, level, last)
        assert adler == zlib.adler32(p.tobytes())
        d = zlib.decompressobj(-15)
        assert d.decompress(part) == p.tobytes()
        assert d.eof == last, "only the final part may end the stream"
        stream += part
        total += p.tobytes()
    d = zlib.decompressobj(-15)
    assert d.decompress(stream) == total and d.eof and d.unused_data == b""
