"""End-to-end PNG encoding, DEFLATE streams and checksums on the GPU.

Every PNG is decoded by the oracle's PNG reader: chunk CRCs are checked with
zlib.crc32, the IDAT stream is inflated by stock zlib (which also checks the
zlib header and the Adler-32 trailer), and the unfiltered pixels must equal
the oracle's windowed pixels.  The filtered scanlines must equal the oracle's
filter output byte for byte.
"""
import zlib

import numpy as np
import pytest

from test_gpu_filter import expected_filtered

pytestmark = pytest.mark.gpu


def decode_and_check(O, r2p, img, raw, png):
    ihdr, pixels, stream, chunks, filt = O.parse_png(png)
    want_filt, win = expected_filtered(O, r2p, img, raw)
    assert ihdr["width"] == img.width and ihdr["height"] == img.height
    assert ihdr["bit_depth"] == 8 * img.out_bytes_per_sample
    assert ihdr["color_type"] == {1: 0, 3: 2, 4: 6}[img.channels]
    assert ihdr["interlace"] == 0
    assert np.array_equal(filt, want_filt), "filtered scanlines differ from the oracle"
    assert np.array_equal(pixels, win), "decoded pixels differ from the oracle"
    flg = {0: 0xDA, 1: 0x01, 2: 0x5E, 5: 0x5E, 6: 0x9C, 7: 0x9C, 8: 0xDA, 9: 0xDA}
    assert stream[0] == 0x78 and stream[1] == flg.get(img.level, stream[1])
    return ihdr, stream


def test_c0_png_stored(engine, O, r2p, W):
    raw = W.ct_phantom(0)
    img = W.image_c0()
    png = engine.encode_png(img, raw)
    decode_and_check(O, r2p, img, raw, png)
    assert len(png) <= r2p.png_bound(img)
    # level 0 stores every filtered byte: 262,656 bytes in 5 stored blocks of 65520
    assert len(png) == 43 + img.filtered_bytes + 5 * 5 + 20


@pytest.mark.parametrize("w,h,ch,bps,mode", [(1, 1, 1, 1, 0), (7, 3, 3, 2, 0), (65520, 1, 1, 1, 0),
                                             (65519, 1, 1, 1, 0), (300, 900, 1, 2, 1), (1000, 70, 4, 1, 0)])
def test_stored_shapes(engine, O, r2p, w, h, ch, bps, mode):
    rng = np.random.default_rng(w + h)
    raw = rng.integers(0, 256, size=w * h * ch * bps, dtype=np.uint8)
    img = r2p.Image.make(w, h, ch, bps, mode, level=0)
    decode_and_check(O, r2p, img, raw, engine.encode_png(img, raw))


def test_device_entry_point(engine, O, r2p, W):
    raw = W.ct_phantom(3, 256, 256)
    img = W.image_ct8(256, 256, -100.0, 700.0, level=0)
    cap = r2p.png_bound(img)
    d_raw = r2p.DeviceBuffer.from_array(raw)
    d_png = r2p.DeviceBuffer(cap)
    d_len = r2p.DeviceBuffer(8)
    engine.encode_png_device(img, d_raw.ptr, d_png.ptr, cap, d_len.ptr)
    n = int(d_len.download(8).view(np.uint64)[0])
    decode_and_check(O, r2p, img, raw, d_png.download(n).tobytes())


def test_batch_stored(engine, O, r2p, W):
    specs = [(256, 256, 40.0, 400.0), (512, 300, -500.0, 90.0), (33, 17, 0.0, 1500.0), (1024, 64, 200.0, 255.0)]
    imgs, raws, bufs, outs, caps = [], [], [], [], []
    for i, (w, h, wc, ww) in enumerate(specs):
        raw = W.ct_phantom(20 + i, w, h)
        img = W.image_ct8(w, h, wc, ww, level=0)
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


@pytest.mark.parametrize("n", [1, 15, 16, 4095, 65519, 65520, 65521, 200003])
def test_zlib_stored_stream(engine, n):
    rng = np.random.default_rng(n)
    data = rng.integers(0, 256, size=n, dtype=np.uint8)
    z = engine.zlib_compress(data, 0)
    assert z[:2] == b"\x78\xda"
    assert zlib.decompress(z) == data.tobytes()


@pytest.mark.parametrize("n", [0, 1, 3, 4, 5, 251, 252, 253, 65535, 65536, 65537, 1000003])
def test_checksums_vs_zlib(engine, n):
    rng = np.random.default_rng(n + 1)
    data = rng.integers(0, 256, size=n, dtype=np.uint8)
    assert engine.checksum(data, "adler32") == zlib.adler32(data.tobytes())
    assert engine.checksum(data, "crc32") == zlib.crc32(data.tobytes())


def test_checksums_all_ones_and_unaligned(engine, r2p):
    data = np.full(300001, 255, np.uint8)
    assert engine.checksum(data, "adler32") == zlib.adler32(data.tobytes())
    assert engine.checksum(data, "crc32") == zlib.crc32(data.tobytes())
    # unaligned device start
    buf = r2p.DeviceBuffer.from_array(np.arange(70000, dtype=np.uint32).view(np.uint8))
    res = r2p.DeviceBuffer(4)
    ref = np.arange(70000, dtype=np.uint32).view(np.uint8)[3:3 + 123457].tobytes()
    engine.crc32_device(buf.ptr + 3, 123457, res.ptr)
    assert int(res.download(4).view(np.uint32)[0]) == zlib.crc32(ref)
    engine.adler32_device(buf.ptr + 3, 123457, res.ptr)
    assert int(res.download(4).view(np.uint32)[0]) == zlib.adler32(ref)


def test_encode_png_many_matches_single_calls(engine, O, r2p, W):
    """r2p_encode_png_many keeps several images in flight; each result equals
    r2p_encode_png of the same image, and one bad image fails alone."""
    specs = [(300, 200, 1, 1), (640, 480, 2, 1), (128, 96, 1, 0), (1024, 700, 2, 6), (77, 33, 1, 1),
             (512, 512, 2, 0), (900, 300, 1, 1), (256, 256, 2, 1), (333, 444, 1, 1)]
    imgs, raws = [], []
    for i, (w, h, kind, level) in enumerate(specs):
        raw = W.ct_phantom(60 + i, w, h)
        img = (W.image_ct8 if kind == 1 else W.image_ct16)(w, h, 40.0 + i, 400.0, level=level)
        imgs.append(img)
        raws.append(raw)
    bad = r2p.Image.make(64, 64, 2, 2, r2p.WINDOW_NONE)          # 2 channels: rejected
    imgs.insert(4, bad)
    raws.insert(4, np.zeros(64 * 64 * 2, np.uint16))
    sts, pngs = engine.encode_png_many(imgs, raws)
    assert sts[4] == r2p.EINVAL and pngs[4] is None
    for i, (img, raw) in enumerate(zip(imgs, raws)):
        if i == 4:
            continue
        assert sts[i] == r2p.OK
        assert pngs[i] == engine.encode_png(img, raw), "image %d differs from the single call" % i
        decode_and_check(O, r2p, img, raw, pngs[i])
    # pinned inputs and a ring of pinned outputs of period 2 * MANY_SLOTS
    pins = []
    for raw in raws[:4]:
        p = r2p.PinnedBuffer(raw.nbytes)
        p.array[:] = raw.view(np.uint8).reshape(-1)
        pins.append(p)
    ring = [r2p.PinnedBuffer(max(r2p.png_bound(im) for im in imgs[:4])) for _ in range(2 * r2p.MANY_SLOTS)]
    n = 3 * len(ring)
    sts, lens = engine.encode_png_many([imgs[i % 4] for i in range(n)], [pins[i % 4] for i in range(n)],
                                       [ring[i % len(ring)] for i in range(n)])
    assert all(st == r2p.OK for st in sts)
    for i in range(n - len(ring), n):                            # the last image written to each buffer
        got = bytes(ring[i % len(ring)].array[:lens[i]])
        assert got == engine.encode_png(imgs[i % 4], raws[i % 4])


def test_encode_png_many_overlapping_downloads(engine, r2p, W):
    """A slot's next upload may run beside its previous PNG download when the
    two regions of the arena do not meet; sizes that change from image to
    image move the regions, and every result must still equal its single
    call (each image has its own pinned output buffer)."""
    sizes = [(1500, 1200), (64, 48), (900, 1700), (1500, 1200), (300, 260), (2048, 700)]
    imgs, raws = [], []
    for i, (w, h) in enumerate(sizes):
        imgs.append(W.image_ct16(w, h, 40.0, 400.0, level=1))
        raws.append(W.ct_phantom(900 + i, w, h))
    order = [(3 * i) % len(sizes) for i in range(4 * len(sizes))] + [0] * 8
    pins = [r2p.PinnedBuffer(raws[j].nbytes) for j in range(len(sizes))]
    for j, p in enumerate(pins):
        p.array[:] = raws[j].view(np.uint8).reshape(-1)
    outs = [r2p.PinnedBuffer(r2p.png_bound(imgs[j])) for j in order]
    sts, lens = engine.encode_png_many([imgs[j] for j in order], [pins[j] for j in order], outs)
    assert all(st == r2p.OK for st in sts)
    single = [engine.encode_png(imgs[j], raws[j]) for j in range(len(sizes))]
    for i, j in enumerate(order):
        assert bytes(outs[i].array[:lens[i]]) == single[j], "image %d (size %s)" % (i, sizes[j])
