"""The C++ host layer's DICOM reader, through `gpu_png_encoder <file> --probe`
(no GPU call): header semantics of the reference's DicomSource::open
(src/dicom_loader.cpp:317-397) and frame bounds of load_frame (:511-531), on
files written by tests/dicom_files.py."""
import json
import os
import subprocess

import numpy as np
import pytest

import dicom_files as D


@pytest.fixture(scope="session")
def cli(r2p):
    import __graft_entry__ as g
    g._load_file("r2p_pkg_build", os.path.join(g.PKG_DIR, "build.py")).build()
    path = os.path.join(g.PKG_DIR, "gpu_png_encoder")
    assert os.access(path, os.X_OK)
    return path


def probe(cli, path):
    r = subprocess.run([cli, str(path), "--probe"], capture_output=True, text=True, timeout=60)
    return r.returncode, (json.loads(r.stdout) if r.returncode == 0 else None), r.stderr


def test_ct_header_explicit(cli, tmp_path):
    px = np.arange(64 * 48, dtype=np.uint16).reshape(48, 64) % 4096
    f = tmp_path / "ct.dcm"
    D.write_dicom(f, px, bits_stored=12, high_bit=11, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0)
    rc, h, err = probe(cli, f)
    assert rc == 0, err
    assert h["transfer_syntax"] == D.EXPLICIT_LE and h["photometric"] == "MONOCHROME2"
    assert (h["width"], h["height"], h["channels"], h["bits_per_sample"], h["bpp"], h["frames"]) == (64, 48, 1, 16, 2, 1)
    assert (h["bits_allocated"], h["bits_stored"], h["high_bit"], h["pixel_rep"]) == (16, 12, 11, 0)
    assert h["apply_rescale"] == 1 and h["rescale_slope"] == 1.0 and h["rescale_intercept"] == -1024.0
    assert h["apply_window"] == 1 and h["window_center"] == 40.0 and h["window_width"] == 400.0


def test_implicit_vr_without_preamble_and_nested_sequences(cli, tmp_path):
    px = np.zeros((3, 20, 30), np.uint16)
    f = tmp_path / "imp.dcm"
    D.write_dicom(f, px, transfer_syntax=D.IMPLICIT_LE, preamble=False, wc="100\\200", ww="300\\400")
    rc, h, err = probe(cli, f)
    assert rc == 0, err
    assert h["transfer_syntax"] == D.IMPLICIT_LE and h["frames"] == 3
    # first value of a multi-valued DS
    assert h["apply_window"] == 1 and h["window_center"] == 100.0 and h["window_width"] == 300.0


def test_rescale_and_window_rules(cli, tmp_path):
    px = np.zeros((8, 8), np.uint16)
    cases = [
        # (slope, intercept, wc, ww) -> (apply_rescale, apply_window)
        ((1.0, 0.0, 40.0, 400.0), (0, 1)),        # identity rescale is not applied
        ((None, -1024.0, None, 400.0), (1, 0)),   # intercept alone; window needs both values
        ((2.0, None, 40.0, 0.0), (1, 0)),         # width 0 disables the window
        ((None, None, None, None), (0, 0)),
    ]
    for i, ((m, b, c, w), want) in enumerate(cases):
        f = tmp_path / ("r%d.dcm" % i)
        D.write_dicom(f, px, slope=m, intercept=b, wc=c, ww=w)
        rc, h, err = probe(cli, f)
        assert rc == 0, err
        assert (h["apply_rescale"], h["apply_window"]) == want, (i, h)
    # HighBit absent -> BitsStored - 1
    f = tmp_path / "hb.dcm"
    D.write_dicom(f, px, bits_stored=10, high_bit=None)
    assert probe(cli, f)[1]["high_bit"] == 9


def test_eight_bit_rgb_and_signed(cli, tmp_path):
    rgb = np.random.default_rng(1).integers(0, 256, size=(1, 10, 12, 3), dtype=np.uint8)
    f = tmp_path / "rgb.dcm"
    D.write_dicom(f, rgb, bits_allocated=8, bits_stored=8, high_bit=7)
    h = probe(cli, f)[1]
    assert (h["channels"], h["bits_per_sample"], h["bpp"]) == (3, 8, 3) and h["photometric"] == "RGB"
    f = tmp_path / "signed.dcm"
    D.write_dicom(f, np.zeros((4, 4), np.uint16), bits_stored=16, high_bit=15, pixel_rep=1)
    assert probe(cli, f)[1]["pixel_rep"] == 1


def test_refusals(cli, tmp_path):
    px = np.zeros((8, 8), np.uint16)
    f = tmp_path / "jpeg.dcm"
    D.write_dicom(f, px, transfer_syntax=D.JPEG_LOSSLESS)
    rc, _, err = probe(cli, f)
    assert rc != 0 and "not supported" in err
    # NumberOfFrames larger than the pixel data holds: load_frame refuses
    f = tmp_path / "short.dcm"
    D.write_dicom(f, px, number_of_frames=2)
    rc, _, err = probe(cli, f)
    assert rc != 0 and "out of range" in err
    # truncated file
    good = tmp_path / "ok.dcm"
    D.write_dicom(good, px)
    data = good.read_bytes()
    f = tmp_path / "trunc.dcm"
    f.write_bytes(data[:-40])
    rc, _, err = probe(cli, f)
    assert rc != 0
    # bits allocated 12 is refused
    f = tmp_path / "b12.dcm"
    D.write_dicom(f, px, bits_allocated=12)
    rc, _, err = probe(cli, f)
    assert rc != 0 and "BitsAllocated" in err


def test_cli_usage_and_unknown_option(cli, tmp_path):
    r = subprocess.run([cli], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "--strip-height" in r.stderr and "--level" in r.stderr
    r = subprocess.run([cli, "a.dcm", "b.png", "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Unknown option" in r.stderr


# --- TIFF ---------------------------------------------------------------------
import tiff_files as T  # noqa: E402


@pytest.mark.parametrize("order", ["II", "MM"])
@pytest.mark.parametrize("shape,dtype", [((33, 41), np.uint16), ((20, 17, 3), np.uint8), ((9, 11, 4), np.uint16)])
def test_tiff_probe(cli, tmp_path, order, shape, dtype):
    rng = np.random.default_rng(7)
    img = rng.integers(0, np.iinfo(dtype).max + 1, size=shape, dtype=dtype)
    f = tmp_path / "a.tif"
    T.write_tiff(f, img, order=order, rows_per_strip=5)
    r = subprocess.run([cli, str(f), "--probe"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    h = json.loads(r.stdout)
    ch = shape[2] if len(shape) == 3 else 1
    assert (h["width"], h["height"], h["channels"], h["bits_per_sample"]) == (shape[1], shape[0], ch, 8 * img.itemsize)
    assert h["rows_read"] == shape[0]
    assert h["byte_sum"] == int(T.expected_png_bytes(img).astype(np.uint64).sum())


def test_tiff_refusals(cli, tmp_path):
    img = np.zeros((8, 8), np.uint16)
    for kw, msg in (({"compression": 5}, "compressed"), ({"tiled": True}, "tiled")):
        f = tmp_path / ("x%s.tif" % msg)
        T.write_tiff(f, img, **kw)
        r = subprocess.run([cli, str(f), "--probe"], capture_output=True, text=True, timeout=60)
        assert r.returncode != 0 and msg in r.stderr
