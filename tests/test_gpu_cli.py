"""gpu_png_encoder and the C++ host layer on the GPU.

Single files follow the reference's single-file pipeline: a DICOM frame keeps
its depth and goes through the DICOM window transform (src/gpu_filter.cu:71-162);
folders follow its batch rules (16-bit grayscale -> 8-bit through the Q15/table
windowing, src/batch_processor.cpp:397-409; multi-frame -> <stem>/slice_NNNN.png).
Every PNG is decoded by the oracle's reader (CRCs, zlib inflate with its
Adler-32 check, unfilter) and compared with the oracle's pixels.
"""
import os
import subprocess
import zlib

import numpy as np
import pytest

import dicom_files as D
from test_host_cli import cli  # noqa: F401  (fixture)

pytestmark = pytest.mark.gpu


def run(cli, *args, timeout=300):
    r = subprocess.run([cli] + [str(a) for a in args], capture_output=True, text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def params(O, bits_stored=12, high_bit=11, pixel_rep=0, slope=None, intercept=None, wc=None, ww=None, ba=16):
    """DicomPixelParams as the reader fills them (rescale/window rules of
    src/dicom_loader.cpp:379-397, which the oracle's make_params applies)."""
    return O.make_params(ba, bits_stored, high_bit, pixel_rep, slope=slope, intercept=intercept, wc=wc, ww=ww)


def check_png(O, path, want_pixels, depth, ctype, max_idat=None):
    data = open(path, "rb").read()
    ihdr, pixels, stream, chunks, filt = O.parse_png(data)
    assert ihdr["bit_depth"] == depth and ihdr["color_type"] == ctype
    assert np.array_equal(pixels, want_pixels), "decoded pixels differ from the oracle"
    if max_idat is not None:
        assert all(n <= max_idat for t, n in chunks if t == b"IDAT")
        assert sum(1 for t, n in chunks if t == b"IDAT") > 1
    return ihdr, filt


@pytest.mark.parametrize("level", [0, 1, 6])
@pytest.mark.parametrize("mode", ["whole", "strips"])
def test_single_dicom16(cli, O, W, tmp_path, level, mode):
    px = W.ct_phantom(3, 300, 257)
    f = tmp_path / "ct.dcm"
    D.write_dicom(f, px, bits_stored=12, high_bit=11, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0)
    out = tmp_path / "ct.png"
    extra = ["--strip-pipeline", "--strip-height", 64, "--idat-chunk", 32768] if mode == "strips" else []
    run(cli, f, out, "--level", level, *extra)
    p = params(O, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0)
    want = O.window_a2(px.view(np.uint8), p)
    _, filt = check_png(O, out, want, 16, 0, 32768 if mode == "strips" else None)
    assert np.array_equal(filt, O.filter_rows(want, 257, 600, 2)), "filtered scanlines differ"


def test_frame_select_all_frames_and_rgb(cli, O, tmp_path):
    rng = np.random.default_rng(9)
    frames = rng.integers(0, 4096, size=(3, 70, 90), dtype=np.uint16)
    f = tmp_path / "multi.dcm"
    D.write_dicom(f, frames, wc=2048.0, ww=4096.0)
    p = params(O, wc=2048.0, ww=4096.0)
    out = tmp_path / "f1.png"
    run(cli, f, out, "--frame", 1, "--level", 1)
    check_png(O, out, O.window_a2(frames[1].view(np.uint8).reshape(-1), p), 16, 0)
    d = tmp_path / "all"
    run(cli, f, d, "--all", "--level", 1, "--gpu-streams", 2)
    for i in range(3):
        check_png(O, d / ("slice_%04d.png" % i), O.window_a2(frames[i].view(np.uint8).reshape(-1), p), 16, 0)
    rgb = rng.integers(0, 256, size=(1, 50, 41, 3), dtype=np.uint8)
    f = tmp_path / "rgb.dcm"
    D.write_dicom(f, rgb, bits_allocated=8, bits_stored=8, high_bit=7)
    out = tmp_path / "rgb.png"
    run(cli, f, out, "--level", 1)
    check_png(O, out, O.window_a2(rgb.reshape(-1), params(O, 8, 7, ba=8)), 8, 2)


def test_folder_batch_rules(cli, O, W, tmp_path):
    src = tmp_path / "in"
    src.mkdir()
    cts = {}
    for k, (w, h, wc, ww) in enumerate([(256, 256, 40.0, 400.0), (300, 199, -600.0, 150.0), (512, 128, 300.0, 1500.0)]):
        px = W.ct_phantom(20 + k, w, h)
        D.write_dicom(src / ("ct%d.dcm" % k), px, slope=1.0, intercept=-1024.0, wc=wc, ww=ww)
        cts["ct%d" % k] = (px, wc, ww)
    frames = np.random.default_rng(3).integers(0, 4096, size=(2, 40, 60), dtype=np.uint16)
    D.write_dicom(src / "multi.dcm", frames, wc=2048.0, ww=4096.0)
    gray8 = np.random.default_rng(4).integers(0, 256, size=(33, 65), dtype=np.uint8)
    D.write_dicom(src / "eight.dcm", gray8, bits_allocated=8, bits_stored=8, high_bit=7)
    (src / "notes.txt").write_text("not an image")
    dst = tmp_path / "out"
    out = run(cli, src, dst, "--level", 1, "--batch-workers", 2)
    assert "5/5 OK" in out
    for name, (px, wc, ww) in cts.items():
        p = O.make_params(16, 12, 11, 0, slope=1.0, intercept=-1024.0, wc=wc, ww=ww)
        want, _ = O.window8(px.view(np.uint8), p)
        check_png(O, dst / (name + ".png"), want, 8, 0)
    p = params(O, wc=2048.0, ww=4096.0)
    for i in range(2):
        check_png(O, dst / "multi" / ("slice_%04d.png" % i), O.window_a2(frames[i].view(np.uint8).reshape(-1), p),
                  16, 0)
    check_png(O, dst / "eight.png", O.window_a2(gray8.reshape(-1), params(O, 8, 7, ba=8)), 8, 0)
    assert not (dst / "notes.png").exists()


def test_bench_deflate(cli):
    out = run(cli, "--bench-deflate", 1000000)
    rows = [l.split() for l in out.splitlines() if l.strip()[:1].isdigit()]
    assert [r[0] for r in rows] == ["0", "1"] and all(float(r[1]) > 0 for r in rows)


@pytest.mark.parametrize("dicom,level", [(True, 1), (False, 0), (False, 6)])
def test_reference_interfaces_from_cpp(cli, O, W, tmp_path, dicom, level):
    """tests/cpp/compat_check.cpp, built against the host headers and
    libr2p_host.so, uses gpu_filter_* (two contexts, prior row threaded by
    hand, host and device inputs) and CompressionBackend::compress_strip as
    the reference's pipeline does; the result must be the oracle's filtered
    bytes and a zlib stream that inflates to them."""
    pkg = os.path.dirname(cli)
    root = os.path.dirname(pkg)
    exe = tmp_path / "compat_check"
    subprocess.run(["g++", "-std=c++17", "-O1", "-o", str(exe), os.path.join(root, "tests", "cpp", "compat_check.cpp"),
                    "-I" + os.path.join(pkg, "host", "include"), "-I" + os.path.join(root, "include"),
                    "-L" + pkg, "-Wl,-rpath," + pkg, "-lr2p_host", "-lr2p", "-lpthread"], check=True, timeout=300)
    if dicom:
        w, h, bpp = 203, 150, 2
        raw = W.ct_phantom(5, w, h).view(np.uint8).reshape(-1)
        win = O.window_a2(raw, O.make_params(16, 12, 11, 0, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0))
    else:
        w, h, bpp = 111, 97, 6
        raw = np.random.default_rng(8).integers(0, 65536, size=(h, w, 3), dtype=np.uint16).astype(">u2")
        raw = raw.view(np.uint8).reshape(-1)
        win = raw
    (tmp_path / "raw.bin").write_bytes(raw.tobytes())
    args = [exe, tmp_path / "raw.bin", w, h, bpp, 32, level, int(dicom), tmp_path / "f.out", tmp_path / "z.out"]
    r = subprocess.run([str(a) for a in args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    filt = np.frombuffer((tmp_path / "f.out").read_bytes(), np.uint8)
    assert np.array_equal(filt, O.filter_rows(win, h, w * bpp, bpp)), "filtered strips differ from the oracle"
    assert zlib.decompress((tmp_path / "z.out").read_bytes()) == filt.tobytes()


import tiff_files as T  # noqa: E402


@pytest.mark.parametrize("order,photo", [("II", None), ("MM", None), ("II", 0)])
def test_tiff_to_png(cli, O, tmp_path, order, photo):
    """TIFF in the reference's loader conventions: 16-bit samples
    big-endian in the PNG, MINISWHITE inverted (src/image_loader.cpp:200-212)."""
    rng = np.random.default_rng(11)
    img = (rng.integers(0, 4096, size=(57, 83, 3)) * 16).astype(np.uint16)
    if photo == 0:
        img = img[..., 0]
    f = tmp_path / "rgb.tif"
    T.write_tiff(f, img, order=order, rows_per_strip=9, photometric=photo)
    out = tmp_path / "rgb.png"
    run(cli, f, out, "--level", 1)
    check_png(O, out, T.expected_png_bytes(img, photo), 16, 2 if img.ndim == 3 else 0)


def test_folder_with_tiff(cli, O, W, tmp_path):
    src = tmp_path / "in"
    src.mkdir()
    img = np.random.default_rng(12).integers(0, 256, size=(40, 50, 3), dtype=np.uint8)
    T.write_tiff(src / "photo.tif", img, rows_per_strip=16)
    px = W.ct_phantom(30, 128, 96)
    D.write_dicom(src / "ct.dcm", px, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0)
    dst = tmp_path / "out"
    out = run(cli, src, dst, "--level", 1)
    assert "2/2 OK" in out
    check_png(O, dst / "photo.png", T.expected_png_bytes(img), 8, 2)
    want, _ = O.window8(px.view(np.uint8), O.make_params(16, 12, 11, 0, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0))
    check_png(O, dst / "ct.png", want, 8, 0)


# ---- BMP export (--format bmp): the reference's BMP path, written on the GPU
def test_bmp_single_files(cli, O, W, tmp_path):
    px = W.ct_phantom(4, 301, 97)
    f = tmp_path / "ct.dcm"
    D.write_dicom(f, px, bits_stored=12, high_bit=11, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0)
    out = tmp_path / "ct.bmp"
    run(cli, f, out, "--format", "bmp", "--all")                    # --all is ignored for BMP
    p = params(O, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0)
    assert out.read_bytes() == O.bmp_file(px.view(np.uint8), 301, 97, 1, 2, "dicom", p)
    rgb = np.random.default_rng(5).integers(0, 65536, size=(23, 37, 3), dtype=np.uint16)
    t = tmp_path / "rgb.tif"
    T.write_tiff(t, rgb, order="MM")
    out = tmp_path / "rgb.bmp"
    run(cli, t, out, "--format", "BMP")
    assert out.read_bytes() == O.bmp_file(T.expected_png_bytes(rgb), 37, 23, 3, 2, "be")


def test_bmp_folder(cli, O, W, tmp_path):
    src, dst = tmp_path / "in", tmp_path / "out"
    src.mkdir()
    ct = W.ct_phantom(6, 128, 96)
    D.write_dicom(src / "a.dcm", ct, bits_stored=12, high_bit=11, slope=1.0, intercept=-1024.0, wc=40.0, ww=100.0)
    u8 = np.random.default_rng(6).integers(0, 256, size=(1, 33, 45), dtype=np.uint8)
    D.write_dicom(src / "b.dcm", u8, bits_allocated=8, bits_stored=8, high_bit=7)
    frames = np.random.default_rng(7).integers(0, 4096, size=(2, 20, 30), dtype=np.uint16)
    D.write_dicom(src / "c.dcm", frames, wc=2048.0, ww=4096.0)
    g = np.random.default_rng(8).integers(0, 65536, size=(17, 29), dtype=np.uint16)
    T.write_tiff(src / "d.tif", g)
    run(cli, src, dst, "--format", "bmp", "--level", 1)
    p = params(O, slope=1.0, intercept=-1024.0, wc=40.0, ww=100.0)
    # 16-bit grayscale: the batch 16->8 rule, then an 8-bit BMP
    assert (dst / "a.bmp").read_bytes() == O.bmp_file(ct.view(np.uint8), 128, 96, 1, 2, "batch8", p)
    assert (dst / "b.bmp").read_bytes() == O.bmp_file(u8.reshape(-1), 45, 33, 1, 1, "dicom",
                                                        params(O, 8, 7, ba=8))
    assert (dst / "d.bmp").read_bytes() == O.bmp_file(T.expected_png_bytes(g), 29, 17, 1, 2, "be")
    # multi-frame files stay PNG slices, as in the reference
    pf = params(O, wc=2048.0, ww=4096.0)
    for i in range(2):
        check_png(O, dst / "c" / ("slice_%04d.png" % i), O.window_a2(frames[i].view(np.uint8).reshape(-1), pf), 16, 0)


def test_strip_pipeline_many_strips(cli, O, W, tmp_path):
    # 33 strips through the three-slot reader ring and the writer thread
    px = W.ct_phantom(11, 173, 263)
    f = tmp_path / "ct.dcm"
    D.write_dicom(f, px, bits_stored=12, high_bit=11, wc=40.0, ww=400.0, slope=1.0, intercept=-1024.0)
    out = tmp_path / "ct.png"
    run(cli, f, out, "--level", 1, "--strip-pipeline", "--strip-height", 8, "--idat-chunk", 4096)
    want = O.window_a2(px.view(np.uint8), params(O, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0))
    _, filt = check_png(O, out, want, 16, 0, 4096)
    assert np.array_equal(filt, O.filter_rows(want, 263, 346, 2))
