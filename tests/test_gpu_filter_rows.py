"""The warp-per-row window + filter kernel (rows of 2048 filtered bytes and
more), bit-exact against the oracle's restatement of the reference
(windowing src/gpu_filter.cu:71-162 and src/batch_processor.cpp:100-266;
filter src/gpu_filter.cu:183-309; prior-row carry src/gpu_filter.cu:391-434).

Every window kind the kernel compiles (16-bit tables with and without a
shift, 8-bit tables, Q15, byte copy and byte swap), every bytes-per-pixel
value (1, 2, 3, 4, 6, 8), rows whose last 16-byte unit is half full, heights
that are not a multiple of the kernel's rows per CTA, and output rows at
every alignment (a row holds rb + 1 bytes), with 256-byte guard zones around
the output that must stay untouched.
"""
import numpy as np
import pytest

from test_gpu_filter import expected_filtered

pytestmark = pytest.mark.gpu

GUARD = 256


def filter_guarded(r2p, engine, img, raw, prior=None):
    n = img.filtered_bytes
    out = r2p.DeviceBuffer.from_array(np.full(n + 2 * GUARD, 0xA5, np.uint8))
    px = r2p.DeviceBuffer.from_array(np.ascontiguousarray(raw).view(np.uint8).reshape(-1))
    pr = r2p.DeviceBuffer.from_array(np.ascontiguousarray(prior, np.uint8)) if prior is not None else None
    engine.window_filter_device(img, px.ptr, out.ptr + GUARD, pr.ptr if pr else None)
    buf = out.download()
    assert np.all(buf[:GUARD] == 0xA5) and np.all(buf[GUARD + n:] == 0xA5), "write outside the filtered rows"
    return buf[GUARD:GUARD + n]


def check_rows(O, r2p, engine, img, raw, prior=None):
    assert img.row_bytes >= 2048
    want, _ = expected_filtered(O, r2p, img, raw, prior)
    got = filter_guarded(r2p, engine, img, raw, prior)
    if not np.array_equal(got, want):
        rb = img.row_bytes + 1
        bad = np.nonzero(got != want)[0]
        r = bad[0] // rb
        raise AssertionError("mismatch at byte %d (row %d col %d, type got %d want %d), %d bytes differ"
                             % (bad[0], r, bad[0] % rb, got[r * rb], want[r * rb], bad.size))
    return want


def mixed_rows(rng, h, nbytes, dtype=np.uint8, hi=256):
    """Rows that favour different filters: smooth ramps, repeated rows,
    noise, flat rows and column-correlated rows."""
    out = np.empty((h, nbytes), dtype)
    base = rng.integers(0, hi, size=nbytes, dtype=np.int64)
    for r in range(h):
        k = r % 5
        if k == 0:
            out[r] = (np.arange(nbytes) * (r + 1) // 7) % hi
        elif k == 1:
            out[r] = base
        elif k == 2:
            out[r] = rng.integers(0, hi, size=nbytes)
        elif k == 3:
            out[r] = (base + r * 3) % hi
        else:
            out[r] = (np.cumsum(rng.integers(-2, 3, size=nbytes)) + hi // 2) % hi
    return out


@pytest.mark.parametrize("w,ch,bps,seed", [
    (4112, 1, 1, 1),      # gray8, bpp 1
    (1376, 3, 1, 2),      # RGB8, bpp 3
    (1040, 4, 1, 3),      # RGBA8, bpp 4
    (2056, 1, 2, 4),      # gray16, bpp 2
    (1368, 3, 2, 5),      # RGB16, bpp 6 (two words back)
    (520, 4, 2, 6),       # RGBA16, bpp 8
    (6000, 3, 2, 7),      # C2's row shape
])
def test_rows_copy_all_bpp(O, r2p, engine, w, ch, bps, seed):
    rng = np.random.default_rng(seed)
    h = 13
    raw = mixed_rows(rng, h, w * ch * bps)
    img = r2p.Image.make(w, h, ch, bps, r2p.WINDOW_NONE)
    want = check_rows(O, r2p, engine, img, raw)
    types = set(want[::img.row_bytes + 1].tolist())
    assert len(types) >= 3, types


def test_rows_swap16(O, r2p, engine):
    rng = np.random.default_rng(8)
    raw = rng.integers(0, 65536, size=(11, 2056), dtype=np.uint16).astype("<u2")
    raw[::3] = raw[0]
    check_rows(O, r2p, engine, r2p.Image.make(2056, 11, 1, 2, r2p.WINDOW_SWAP16), raw)


@pytest.mark.parametrize("high_bit,wc,ww", [(11, 2048.0, 4096.0), (11, 1500.0, 800.0), (15, 30000.0, 50000.0)])
def test_rows_dicom16_tables(O, r2p, engine, W, high_bit, wc, ww):
    # 12 bits stored at the bottom (table indexed by the masked sample) or
    # at the top of the word (shifted index)
    w, h = 3072, 19
    raw = W.radial_rects(3, w, h).astype(np.uint32)
    if high_bit == 15:
        raw = raw << 4
    raw = raw.astype("<u2")
    dp = r2p.DicomParams.make(16, 12, high_bit, 0, wc=wc, ww=ww)
    check_rows(O, r2p, engine, r2p.Image.make(w, h, 1, 2, r2p.WINDOW_DICOM16, dp), raw)


def test_rows_dicom16_signed_rescaled(O, r2p, engine):
    rng = np.random.default_rng(9)
    raw = rng.integers(0, 4096, size=(10, 2064), dtype=np.uint16).astype("<u2")
    dp = r2p.DicomParams.make(16, 12, 11, 1, slope=1.5, intercept=-100.0, wc=40.0, ww=700.0)
    check_rows(O, r2p, engine, r2p.Image.make(2064, 10, 1, 2, r2p.WINDOW_DICOM16, dp), raw)


def test_rows_dicom16_8bit_samples(O, r2p, engine):
    rng = np.random.default_rng(10)
    raw = mixed_rows(rng, 9, 4128)
    dp = r2p.DicomParams.make(8, 8, 7, 0, wc=100.0, ww=120.0)
    check_rows(O, r2p, engine, r2p.Image.make(4128, 9, 1, 1, r2p.WINDOW_DICOM16, dp), raw)


@pytest.mark.parametrize("w,wc,ww", [(4104, 40.0, 400.0), (4104, 60.0, 150.0), (5000, -600.0, 1500.0),
                                     (2048, 40.0, 400.0), (3072, -100.0, 700.0), (2056, 60.0, 150.0)])
def test_rows_batch8(O, r2p, engine, W, w, wc, ww):
    # 16-bit samples to 8-bit rows: Q15 (WW 400, 1500, 700) or the FP32 table
    # (WW 150); 4104 and 2056 leave a half unit at each row's end; 2048 and
    # 3072 are the CT batch's two largest slice widths
    h = 17
    raw = W.ct_phantom(11, w, h)
    img = W.image_ct8(w, h, wc, ww)
    check_rows(O, r2p, engine, img, raw)


def test_rows_prior_row(O, r2p, engine):
    rng = np.random.default_rng(12)
    raw = mixed_rows(rng, 7, 4160)
    prior = rng.integers(0, 256, size=4160, dtype=np.uint8)
    check_rows(O, r2p, engine, r2p.Image.make(4160, 7, 1, 1, r2p.WINDOW_NONE), raw, prior)


@pytest.mark.parametrize("mode", ["a2", "batch8", "none_rgb16"])
def test_rows_strips_with_carried_last_row(O, r2p, engine, W, mode):
    """Strips of a wide image with the windowed last row carried from strip
    to strip equal the whole image filtered at once."""
    if mode == "a2":
        w, h = 2056, 45
        raw = W.radial_rects(5, w, h)
        full = r2p.Image.make(w, h, 1, 2, r2p.WINDOW_DICOM16,
                              r2p.DicomParams.make(16, 12, 11, 0, wc=1500.0, ww=3000.0))
    elif mode == "batch8":
        w, h = 4104, 45
        raw = W.ct_phantom(6, w, h)
        full = W.image_ct8(w, h, 40.0, 400.0)
    else:
        w, h = 1368, 45
        raw = np.random.default_rng(6).integers(0, 65536, size=(h, w, 3), dtype=np.uint16).astype(">u2")
        full = r2p.Image.make(w, h, 3, 2, r2p.WINDOW_NONE)
    want, win = expected_filtered(O, r2p, full, raw)
    rb = full.row_bytes
    raw8 = np.ascontiguousarray(raw).view(np.uint8).reshape(h, -1)
    prior = None
    keep = []
    parts = []
    for r0 in range(0, h, 11):
        n = min(11, h - r0)
        img = r2p.Image.make(w, n, full.channels, full.bytes_per_sample, full.window_mode, full.dicom)
        d_raw = r2p.DeviceBuffer.from_array(np.ascontiguousarray(raw8[r0:r0 + n]))
        d_out = r2p.DeviceBuffer(img.filtered_bytes + 16)
        new_last = r2p.DeviceBuffer(rb)
        engine.window_filter_device(img, d_raw.ptr, d_out.ptr, d_prior=prior, d_last_row=new_last.ptr)
        parts.append(d_out.download(img.filtered_bytes))
        assert np.array_equal(new_last.download(rb), win.reshape(h, rb)[r0 + n - 1]), "carried row differs"
        keep.append(new_last)
        prior = new_last.ptr
    assert np.array_equal(np.concatenate(parts), want)


def test_rows_png_and_batch_mixed_widths(O, r2p, engine, W):
    """Wide images (this kernel) and narrow ones (the register-group kernel)
    in one batch give the bytes each gives alone, and decode to the oracle's
    pixels."""
    from test_gpu_png import decode_and_check
    imgs, raws = [], []
    for k, (w, h) in enumerate([(2056, 40), (300, 50), (3072, 33), (640, 20), (4104, 25)]):
        if k % 2 == 0 and w != 4104:
            raws.append(W.radial_rects(k, w, h))
            imgs.append(r2p.Image.make(w, h, 1, 2, r2p.WINDOW_DICOM16,
                                       r2p.DicomParams.make(16, 12, 11, 0, wc=2048.0, ww=4096.0), level=1))
        else:
            raws.append(W.ct_phantom(k, w, h))
            imgs.append(W.image_ct8(w, h, 40.0, 400.0, level=1))
    alone = [engine.encode_png(img, raw) for img, raw in zip(imgs, raws)]
    for img, raw, png in zip(imgs, raws, alone):
        decode_and_check(O, r2p, img, raw, png)
    bufs = [r2p.DeviceBuffer.from_array(raw) for raw in raws]
    caps = [r2p.png_bound(img) for img in imgs]
    outs = [r2p.DeviceBuffer(c) for c in caps]
    lens = r2p.DeviceBuffer(8 * len(imgs))
    engine.encode_batch_device(imgs, [b.ptr for b in bufs], [o.ptr for o in outs], caps, lens.ptr)
    ln = lens.download(8 * len(imgs)).view(np.uint64)
    batch = [outs[i].download(int(ln[i])).tobytes() for i in range(len(imgs))]
    assert batch == [bytes(a) for a in alone]
