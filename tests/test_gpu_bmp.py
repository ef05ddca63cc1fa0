"""BMP export on the GPU (r2p_encode_bmp / r2p_encode_bmp_device).

Every file must equal, byte for byte, the BMP the reference's own export
wrote for the same pixels (tests/golden/bmp_ref.npz, see test_oracle.py) and
the oracle's restatement of it at sizes the fixtures do not cover.
"""
import numpy as np
import pytest

from test_oracle import bmp_golden

pytestmark = pytest.mark.gpu

MODE = {"dicom": "WINDOW_DICOM16", "be": "WINDOW_NONE", "batch8": "WINDOW_BATCH8"}


def r2p_params(r2p, p):
    dp = r2p.DicomParams()
    for k, _ in dp._fields_:
        setattr(dp, k, getattr(p, k))
    return dp


def bmp_image(r2p, m, p):
    return r2p.Image.make(m["width"], m["height"], m["channels"], m["bytes_per_sample"], getattr(r2p, MODE[m["mode"]]),
                          r2p_params(r2p, p) if p is not None else None)


def test_bmp_matches_reference_export(engine, O, r2p):
    for m, p, raw, want in bmp_golden(O):
        img = bmp_image(r2p, m, p)
        assert r2p.bmp_bound(img) == len(want), m["name"]
        assert engine.encode_bmp(img, raw) == want, m["name"]


def test_bmp_device_entry_point(engine, O, r2p):
    stream = r2p.Stream()
    for m, p, raw, want in bmp_golden(O)[:6]:
        img = bmp_image(r2p, m, p)
        cap = r2p.bmp_bound(img)
        d_raw = r2p.DeviceBuffer.from_array(raw)
        d_bmp = r2p.DeviceBuffer(cap + 64)
        engine.encode_bmp_device(img, d_raw.ptr, d_bmp.ptr, cap, stream)
        stream.sync()
        assert d_bmp.download(cap).tobytes() == want, m["name"]


@pytest.mark.parametrize("w,h,ch", [(1, 1, 1), (7, 3, 1), (5, 4, 3), (6, 2, 4), (97, 13, 3)])
def test_bmp_little_endian_16bit(engine, O, r2p, w, h, ch):
    raw = np.random.default_rng(w * 100 + h).integers(0, 256, w * h * ch * 2, dtype=np.uint8)
    img = r2p.Image.make(w, h, ch, 2, r2p.WINDOW_SWAP16)
    assert engine.encode_bmp(img, raw) == O.bmp_file(raw, w, h, ch, 2, "le")


@pytest.mark.parametrize("seed", range(4))
def test_bmp_random_windows(engine, O, r2p, seed):
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(1, 300)), int(rng.integers(1, 60))
    bs = int(rng.choice([10, 12, 16]))
    rep = int(rng.integers(0, 2))
    wc, ww = float(rng.uniform(-1000, 3000)), float(rng.uniform(0.5, 5000))
    slope, icpt = float(rng.choice([1.0, 0.5, 2.0])), float(rng.choice([0.0, -1024.0, 100.0]))
    raw = rng.integers(0, 1 << bs, w * h).astype("<u2").view(np.uint8)
    p = O.make_params(16, bs, None, rep, slope, icpt, wc, ww)
    img = r2p.Image.make(w, h, 1, 2, r2p.WINDOW_DICOM16, r2p_params(r2p, p))
    assert engine.encode_bmp(img, raw) == O.bmp_file(raw, w, h, 1, 2, "dicom", p)
    img8 = r2p.Image.make(w, h, 1, 2, r2p.WINDOW_BATCH8, r2p_params(r2p, p))
    assert engine.encode_bmp(img8, raw) == O.bmp_file(raw, w, h, 1, 2, "batch8", p)


def test_bmp_full_size_c1(engine, O, r2p, W):
    # the 3072x3072 16-bit workload, exported through the BMP formula
    raw = W.radial_rects(1, 3072, 3072)
    p = O.make_params(16, 12, None, 0, None, None, 2048.0, 4096.0)
    img = r2p.Image.make(3072, 3072, 1, 2, r2p.WINDOW_DICOM16, r2p_params(r2p, p))
    got = engine.encode_bmp(img, raw)
    assert len(got) == 1078 + 3072 * 3072
    assert got == O.bmp_file(raw.view(np.uint8), 3072, 3072, 1, 2, "dicom", p)


def test_bmp_rejects(engine, r2p):
    img = r2p.Image.make(8, 8, 4, 1, r2p.WINDOW_NONE)              # 8-bit RGBA
    assert r2p.bmp_bound(img) == 0
    with pytest.raises(r2p.R2PError):
        engine.encode_bmp(img, np.zeros(8 * 8 * 4, np.uint8))
    ok = r2p.Image.make(8, 8, 1, 1, r2p.WINDOW_NONE)
    cap = r2p.bmp_bound(ok)
    d_raw = r2p.DeviceBuffer(64)
    d_bmp = r2p.DeviceBuffer(cap + 64)
    with pytest.raises(r2p.R2PError):                               # output not 4-byte aligned
        engine.encode_bmp_device(ok, d_raw.ptr, d_bmp.ptr + 2, cap)
    with pytest.raises(r2p.R2PError):                               # capacity below the file size
        engine.encode_bmp_device(ok, d_raw.ptr, d_bmp.ptr, cap - 1)
