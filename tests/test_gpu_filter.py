"""Window + adaptive filter on the GPU, bit-exact against the oracle.

Each case runs r2p_window_filter_device (C ABI) and compares the filtered
scanlines -- filter-type bytes and filtered bytes -- with the CPU oracle's
restatement of the reference (windowing src/gpu_filter.cu:71-162 and
src/batch_processor.cpp:100-266; filter src/gpu_filter.cu:183-309).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def expected_filtered(O, r2p, img, raw, prior=None):
    raw8 = np.ascontiguousarray(raw).view(np.uint8).reshape(-1)
    p = O.OrcParams.from_buffer_copy(bytes(img.dicom))
    if img.window_mode == r2p.WINDOW_BATCH8:
        win, _ = O.window8(raw8, p)
    elif img.window_mode == r2p.WINDOW_DICOM16:
        win = O.window_a2(raw8, p)
    elif img.window_mode == r2p.WINDOW_SWAP16:
        win = raw8.reshape(-1, 2)[:, ::-1].reshape(-1).copy()
    else:
        win = raw8
    rb = img.row_bytes
    bpp = img.channels * img.out_bytes_per_sample
    return O.filter_rows(win, img.height, rb, bpp, prior), win


def check(engine, O, r2p, img, raw, prior=None):
    want, win = expected_filtered(O, r2p, img, raw, prior)
    got = engine.filter_image(img, raw, prior)
    if not np.array_equal(got, want):
        rb = img.row_bytes + 1
        bad = np.nonzero(got != want)[0]
        r = bad[0] // rb
        raise AssertionError("mismatch at byte %d (row %d col %d, type got %d want %d), %d bytes differ"
                             % (bad[0], r, bad[0] % rb, got[r * rb], want[r * rb], bad.size))
    return want


def test_c0_q15(engine, O, r2p, W):
    raw = W.ct_phantom(0)
    img = W.image_c0()
    p = O.OrcParams.from_buffer_copy(bytes(img.dicom))
    assert O.q15_coeffs(p) is not None          # WW 400 takes the Q15 path
    check(engine, O, r2p, img, raw)


@pytest.mark.parametrize("ww", [150.0, 80.0, 254.0])
def test_batch8_lut_narrow_window(engine, O, r2p, W, ww):
    raw = W.ct_phantom(1, 300, 211)
    img = W.image_ct8(300, 211, 60.0, ww)
    assert O.q15_coeffs(O.OrcParams.from_buffer_copy(bytes(img.dicom))) is None   # table fallback
    check(engine, O, r2p, img, raw)


def test_batch8_shifted_and_signed(engine, O, r2p, W):
    rng = np.random.default_rng(5)
    raw = rng.integers(0, 65536, size=(97, 130), dtype=np.uint16).astype("<u2")
    for hb, pr in ((15, 0), (11, 1), (15, 1)):
        p = r2p.DicomParams.make(16, 12, hb, pr, slope=1.5, intercept=-300.0, wc=100.0, ww=900.0)
        img = r2p.Image.make(130, 97, 1, 2, r2p.WINDOW_BATCH8, p)
        check(engine, O, r2p, img, raw)


def test_batch8_no_window(engine, O, r2p):
    rng = np.random.default_rng(6)
    raw = rng.integers(0, 4096, size=(64, 64), dtype=np.uint16).astype("<u2")
    for pr in (0, 1):
        p = r2p.DicomParams.make(16, 12, 11, pr)
        img = r2p.Image.make(64, 64, 1, 2, r2p.WINDOW_BATCH8, p)
        check(engine, O, r2p, img, raw)


def test_dicom16_lut(engine, O, r2p, W):
    raw = W.radial_rects(1, 320, 200)
    img = r2p.Image.make(320, 200, 1, 2, r2p.WINDOW_DICOM16, r2p.DicomParams.make(16, 12, 11, 0, wc=2048.0, ww=4096.0))
    check(engine, O, r2p, img, raw)


def test_dicom16_direct_signed_rescale(engine, O, r2p):
    rng = np.random.default_rng(7)
    raw = rng.integers(0, 65536, size=(50, 77), dtype=np.uint16).astype("<u2")
    p = r2p.DicomParams.make(16, 16, 15, 1, slope=0.7, intercept=-100.0, wc=30.0, ww=2500.0)
    img = r2p.Image.make(77, 50, 1, 2, r2p.WINDOW_DICOM16, p)
    check(engine, O, r2p, img, raw)
    p = r2p.DicomParams.make(16, 14, 15, 0, slope=2.0, wc=900.0, ww=0.5)   # step function (w-1 <= 0)
    img = r2p.Image.make(77, 50, 1, 2, r2p.WINDOW_DICOM16, p)
    check(engine, O, r2p, img, raw)


def test_dicom16_8bit_input(engine, O, r2p):
    rng = np.random.default_rng(8)
    raw = rng.integers(0, 256, size=(40, 99), dtype=np.uint8)
    p = r2p.DicomParams.make(8, 8, 7, 1, slope=1.0, intercept=5.0, wc=10.0, ww=120.0)
    img = r2p.Image.make(99, 40, 1, 1, r2p.WINDOW_DICOM16, p)
    check(engine, O, r2p, img, raw)


def test_rgb16_unaligned_rows(engine, O, r2p, W):
    raw = W.rgb_sinusoids(2, 257, 33)
    img = r2p.Image.make(257, 33, 3, 2, r2p.WINDOW_NONE)
    check(engine, O, r2p, img, raw)


def test_rgb16_c2_shape_rows(engine, O, r2p, W):
    raw = W.rgb_sinusoids(3, 6000, 24)
    img = r2p.Image.make(6000, 24, 3, 2, r2p.WINDOW_NONE)
    check(engine, O, r2p, img, raw)


def test_rgba8_and_swap16(engine, O, r2p):
    rng = np.random.default_rng(9)
    raw = rng.integers(0, 256, size=(31, 45, 4), dtype=np.uint8)
    check(engine, O, r2p, r2p.Image.make(45, 31, 4, 1, r2p.WINDOW_NONE), raw)
    raw16 = rng.integers(0, 65536, size=(29, 51), dtype=np.uint16).astype("<u2")
    check(engine, O, r2p, r2p.Image.make(51, 29, 1, 2, r2p.WINDOW_SWAP16), raw16)


@pytest.mark.parametrize("w,h", [(1, 1), (1, 7), (2, 3), (3, 1), (5, 9), (17, 4), (4097, 3), (8193, 2)])
def test_ragged_sizes(engine, O, r2p, w, h):
    rng = np.random.default_rng(w * 31 + h)
    raw = rng.integers(0, 256, size=(h, w), dtype=np.uint8)
    check(engine, O, r2p, r2p.Image.make(w, h, 1, 1, r2p.WINDOW_NONE), raw)


def test_widest_row(engine, O, r2p):
    # 17043-pixel RGB16 rows, the widest image the reference describes
    rng = np.random.default_rng(10)
    raw = rng.integers(0, 65536, size=(3, 17043, 3), dtype=np.uint16).astype(">u2")
    check(engine, O, r2p, r2p.Image.make(17043, 3, 3, 2, r2p.WINDOW_NONE), raw)


def test_prior_row(engine, O, r2p):
    # strip semantics: the caller's windowed row above row 0
    rng = np.random.default_rng(11)
    raw = rng.integers(0, 256, size=(9, 300), dtype=np.uint8)
    prior = rng.integers(0, 256, size=300, dtype=np.uint8)
    check(engine, O, r2p, r2p.Image.make(300, 9, 1, 1, r2p.WINDOW_NONE), raw, prior)


def test_all_filter_types_chosen(engine, O, r2p, W):
    # a mixed image whose rows pick every one of the five filters
    raw = W.rgb_sinusoids(4, 640, 64)
    img = r2p.Image.make(640, 64, 3, 2, r2p.WINDOW_NONE)
    want = check(engine, O, r2p, img, raw)
    rng = np.random.default_rng(12)
    noise = rng.integers(0, 256, size=(64, 640), dtype=np.uint8)
    noise[::4] = 7
    want2 = check(engine, O, r2p, r2p.Image.make(640, 64, 1, 1, r2p.WINDOW_NONE), noise)
    types = set(want[::img.row_bytes + 1]) | set(want2[::641])
    assert len(types) >= 3


def test_random_fuzz(engine, O, r2p):
    rng = np.random.default_rng(13)
    for _ in range(12):
        w = int(rng.integers(1, 900))
        h = int(rng.integers(1, 60))
        mode = int(rng.integers(0, 4))
        if mode == r2p.WINDOW_BATCH8:
            p = r2p.DicomParams.make(16, 12, 11, int(rng.integers(0, 2)), slope=1.0, intercept=-1024.0,
                                     wc=float(rng.uniform(-600, 400)), ww=float(rng.uniform(80, 1600)))
            img = r2p.Image.make(w, h, 1, 2, mode, p)
            raw = rng.integers(0, 4096, size=(h, w), dtype=np.uint16).astype("<u2")
        elif mode == r2p.WINDOW_DICOM16:
            p = r2p.DicomParams.make(16, 12, 11, 0, wc=float(rng.uniform(0, 4096)), ww=float(rng.uniform(2, 4096)))
            img = r2p.Image.make(w, h, 1, 2, mode, p)
            raw = rng.integers(0, 4096, size=(h, w), dtype=np.uint16).astype("<u2")
        else:
            ch = int(rng.choice([1, 3, 4]))
            bps = int(rng.integers(1, 3)) if mode == r2p.WINDOW_NONE else 2
            img = r2p.Image.make(w, h, ch, bps, mode)
            raw = rng.integers(0, 256, size=w * h * ch * bps, dtype=np.uint8)
        check(engine, O, r2p, img, raw)


@pytest.mark.parametrize("mode", ["a2", "batch8", "none_rgb16"])
def test_strips_with_carried_last_row(engine, O, r2p, W, mode):
    """Strip-by-strip filtering with the windowed last row carried between
    strips (r2p_window_filter_device_ex) equals filtering the whole image, as
    the reference's per-strip prior-row carry does (src/gpu_filter.cu:428-434)."""
    w, h, strip = 257, 203, 64
    if mode == "a2":
        raw = W.radial_rects(4, w, h)
        full = r2p.Image.make(w, h, 1, 2, r2p.WINDOW_DICOM16, r2p.DicomParams.make(16, 12, 11, 0, wc=1500.0,
                                                                                   ww=3000.0))
    elif mode == "batch8":
        raw = W.ct_phantom(4, w, h)
        full = W.image_ct8(w, h, 40.0, 400.0)
    else:
        raw = np.random.default_rng(4).integers(0, 65536, size=(h, w, 3), dtype=np.uint16).astype(">u2")
        full = r2p.Image.make(w, h, 3, 2, r2p.WINDOW_NONE)
    want, win = expected_filtered(O, r2p, full, raw)
    rb = full.row_bytes
    raw8 = np.ascontiguousarray(raw).view(np.uint8).reshape(h, -1)
    last = r2p.DeviceBuffer(rb)
    prior = None
    parts = []
    for r0 in range(0, h, strip):
        n = min(strip, h - r0)
        img = r2p.Image.make(w, n, full.channels, full.bytes_per_sample, full.window_mode, full.dicom)
        d_raw = r2p.DeviceBuffer.from_array(np.ascontiguousarray(raw8[r0:r0 + n]))
        d_out = r2p.DeviceBuffer(img.filtered_bytes + 16)
        new_last = r2p.DeviceBuffer(rb)
        engine.window_filter_device(img, d_raw.ptr, d_out.ptr, d_prior=prior, d_last_row=new_last.ptr)
        parts.append(d_out.download(img.filtered_bytes))
        got_last = new_last.download(rb)
        assert np.array_equal(got_last, win.reshape(h, rb)[r0 + n - 1]), "carried row differs from the oracle"
        last = new_last
        prior = last.ptr
    assert np.array_equal(np.concatenate(parts), want)


def _golden():
    import os
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gpu_filter_ref.npz"))


_SPLIT = {1: (1, 1), 2: (1, 2), 3: (3, 1), 4: (4, 1), 6: (3, 2), 8: (4, 2)}


def test_pinned_to_reference_kernels(engine, O, r2p):
    """The fused window+filter kernel against outputs of the reference's own
    dicom_preprocess_kernel + filter_select_kernel (src/gpu_filter.cu, IEEE
    build) recorded on a GB300 (tests/golden/gen_gpu_golden.py)."""
    d = _golden()
    for k in range(int(d["n_flt"][0])):
        wpx, rows, bpp = (int(x) for x in d["flt_%d_meta" % k])
        prior = d["flt_%d_prior" % k]
        pb = d["flt_%d_params" % k]
        if pb.size:
            p = r2p.DicomParams.from_buffer_copy(pb.tobytes())
            bps = p.bits_allocated // 8
            img = r2p.Image.make(wpx, rows, bpp // bps, bps, r2p.WINDOW_DICOM16, p)
        else:
            ch, bps = _SPLIT[bpp]
            img = r2p.Image.make(wpx, rows, ch, bps, r2p.WINDOW_NONE)
        got = engine.filter_image(img, d["flt_%d_in" % k], prior if prior.size else None)
        assert np.array_equal(got, d["flt_%d_ieee" % k]), "case %d differs from the reference kernel" % k
    # every stored value of each window parameter set, as an image
    for k in range(int(d["n_a2"][0])):
        p = r2p.DicomParams.from_buffer_copy(d["a2_%d_params" % k].tobytes())
        ref = d["a2_%d_ieee" % k]
        if p.bits_allocated == 16:
            raw, w, h = np.arange(65536, dtype="<u2"), 256, 256
        else:
            raw, w, h = np.arange(256, dtype=np.uint8), 16, 16
        bps = p.bits_allocated // 8
        img = r2p.Image.make(w, h, 1, bps, r2p.WINDOW_DICOM16, p)
        got = engine.filter_image(img, raw)
        assert np.array_equal(got, O.filter_rows(ref, h, w * bps, bps)), "a2 set %d" % k


@pytest.mark.parametrize("w,h,ch,bps,mode", [(17043, 6, 3, 2, 0), (45000, 5, 1, 2, 2), (13001, 4, 4, 2, 0)])
def test_wide_rows(engine, O, r2p, w, h, ch, bps, mode):
    """Rows too wide to stage next to the ring (>= 90 KB) take the plain-load
    path; the reference handles 17043-pixel RGB16 rows."""
    rng = np.random.default_rng(w)
    raw = rng.integers(0, 4096, size=w * h * ch, dtype=np.uint16).astype("<u2" if mode else ">u2")
    dp = r2p.DicomParams.make(16, 12, 11, 0, wc=2048.0, ww=4096.0) if mode else None
    img = r2p.Image.make(w, h, ch, bps, mode, dp, level=1)
    check(engine, O, r2p, img, raw)
    from test_gpu_png import decode_and_check
    decode_and_check(O, r2p, img, raw, engine.encode_png(img, raw))
