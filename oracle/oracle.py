"""Python face of the oracle -- TEST INFRASTRUCTURE ONLY.

ctypes bindings for oracle/liboracle.so (the CPU restatement of the
reference's window/filter arithmetic and of its zlib encode path), the
reference harnesses in oracle/_ref (where they were built), and a PNG decoder
(chunk walk + CRC check + zlib inflate + PNG unfilter).  Only tests/,
__graft_entry__.smoke() and the CPU-baseline leg of bench.py import this.
"""
import ctypes
import os
import struct
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_u8p = ctypes.POINTER(ctypes.c_uint8)


class OrcParams(ctypes.Structure):
    """Mirror of DicomPixelParams (include/dicom_params.h:6-21)."""
    _fields_ = [
        ("bits_allocated", ctypes.c_int),
        ("bits_stored", ctypes.c_int),
        ("high_bit", ctypes.c_int),
        ("pixel_rep", ctypes.c_int),
        ("apply_rescale", ctypes.c_int),
        ("rescale_slope", ctypes.c_float),
        ("rescale_intercept", ctypes.c_float),
        ("apply_window", ctypes.c_int),
        ("window_center", ctypes.c_float),
        ("window_width", ctypes.c_float),
    ]


def make_params(bits_allocated=16, bits_stored=16, high_bit=None, pixel_rep=0,
                slope=None, intercept=None, wc=None, ww=None):
    """DicomPixelParams the way src/dicom_loader.cpp:372-397 fills them:
    rescale only when slope != 1 or intercept != 0, window only when WW > 0."""
    p = OrcParams()
    p.bits_allocated = bits_allocated
    p.bits_stored = bits_stored
    p.high_bit = bits_stored - 1 if high_bit is None else high_bit
    p.pixel_rep = pixel_rep
    p.rescale_slope, p.rescale_intercept = 1.0, 0.0
    if slope is not None or intercept is not None:
        s = 1.0 if slope is None else slope
        b = 0.0 if intercept is None else intercept
        if abs(s - 1.0) > 1e-9 or abs(b) > 1e-9:
            p.apply_rescale = 1
            p.rescale_slope, p.rescale_intercept = s, b
    p.window_center, p.window_width = 32768.0, 65536.0
    if wc is not None and ww is not None and ww > 0:
        p.apply_window = 1
        p.window_center, p.window_width = wc, ww
    return p


def _ptr(a):
    return a.ctypes.data_as(_u8p)


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            from . import build_oracle  # noqa: F401  (package-relative use)
        L = ctypes.CDLL(path)
        P = ctypes.POINTER(OrcParams)
        L.orc_window_a2.argtypes = [_u8p, ctypes.c_size_t, P, _u8p]
        L.orc_window8.argtypes = [_u8p, ctypes.c_size_t, P, _u8p]
        L.orc_window8.restype = ctypes.c_int
        L.orc_window_q15.argtypes = [_u8p, ctypes.c_size_t, P, _u8p]
        L.orc_window_q15.restype = ctypes.c_int
        L.orc_q15_coeffs.argtypes = [P, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]
        L.orc_q15_coeffs.restype = ctypes.c_int
        L.orc_build_lut.argtypes = [_u8p, P, ctypes.c_int]
        L.orc_bmp_gray8.argtypes = [_u8p, ctypes.c_size_t, P, _u8p]
        L.orc_filter_rows.argtypes = [_u8p, _u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _u8p]
        L.orc_unfilter.argtypes = [_u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, _u8p]
        L.orc_unfilter.restype = ctypes.c_int
        L.port_encoder_create.argtypes = [ctypes.c_int]
        L.port_encoder_create.restype = ctypes.c_void_p
        L.port_encoder_destroy.argtypes = [ctypes.c_void_p]
        L.port_png_from_filtered.argtypes = [ctypes.c_void_p, _u8p, ctypes.c_uint32, ctypes.c_uint32,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, _u8p, ctypes.c_size_t]
        L.port_png_from_filtered.restype = ctypes.c_size_t
        L.port_encode_png.argtypes = [ctypes.c_void_p, _u8p, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_int,
                                      ctypes.c_int, _u8p, ctypes.c_size_t, _u8p]
        L.port_encode_png.restype = ctypes.c_size_t
        _lib = L
    return _lib


# ---------------------------------------------------------------- windowing
def window_a2(raw, p):
    """16-bit-output window (src/gpu_filter.cu:71-162).  raw: uint8 LE bytes
    (bits_allocated 16) or uint8 samples (bits_allocated 8)."""
    raw = np.ascontiguousarray(raw, dtype=np.uint8).reshape(-1)
    n = raw.size // (2 if p.bits_allocated == 16 else 1)
    out = np.empty(raw.size, np.uint8)
    lib().orc_window_a2(_ptr(raw), n, ctypes.byref(p), _ptr(out))
    return out


def window8(raw_le, p):
    """8-bit-output window with the batch dispatch (src/batch_processor.cpp:397-409).
    Returns (pixels, path) where path is 1 for Q15 and 2 for the LUT."""
    raw_le = np.ascontiguousarray(raw_le, dtype=np.uint8).reshape(-1)
    out = np.empty(raw_le.size // 2, np.uint8)
    path = lib().orc_window8(_ptr(raw_le), out.size, ctypes.byref(p), _ptr(out))
    return out, path


def q15_coeffs(p):
    a, b = ctypes.c_int32(), ctypes.c_int32()
    ok = lib().orc_q15_coeffs(ctypes.byref(p), ctypes.byref(a), ctypes.byref(b))
    return (a.value, b.value) if ok else None


def build_lut(p):
    n = 1 << p.bits_stored
    lut = np.empty(n, np.uint8)
    lib().orc_build_lut(_ptr(lut), ctypes.byref(p), n)
    return lut


# ---------------------------------------------------------------------- BMP
def bmp_gray8(raw_le, p):
    """BMP export window (src/pipeline.cpp:1894-1932): 16-bit LE -> 8-bit."""
    raw_le = np.ascontiguousarray(raw_le, dtype=np.uint8).reshape(-1)
    out = np.empty(raw_le.size // 2, np.uint8)
    lib().orc_bmp_gray8(_ptr(raw_le), out.size, ctypes.byref(p), _ptr(out))
    return out


def bmp_file(raw, width, height, channels, bytes_per_sample, mode, p=None):
    """Whole BMP file of an image as the reference's BMP export writes it
    (run_bmp_from_source src/pipeline.cpp:1944-2004; BmpWriter
    src/bmp_writer.cpp:36-131).  mode: 'dicom' (a DICOM source), 'batch8'
    (the folder batch's 16->8 rule, src/batch_processor.cpp:389-422), 'be'
    (16-bit big-endian samples, e.g. TIFF/RAW) or 'le' (16-bit little-endian
    samples: the high byte is second)."""
    raw = np.ascontiguousarray(raw, dtype=np.uint8).reshape(-1)
    oc = 1 if channels == 1 else 3
    if mode == "batch8":
        px, _ = window8(raw, p)
        px = px.reshape(height, width, 1)
    elif mode == "dicom" and bytes_per_sample == 2 and channels == 1:
        px = bmp_gray8(raw, p).reshape(height, width, 1)
    elif bytes_per_sample == 2:
        s = raw.reshape(height, width, channels, 2)[..., 1 if mode == "le" else 0]
        px = s[..., :oc]
    else:
        px = raw.reshape(height, width, channels)[..., :oc]
    if oc == 3:
        px = px[..., ::-1]                                   # RGB -> BGR
    stride = (width * oc + 3) & ~3
    rows = np.zeros((height, stride), np.uint8)
    rows[:, :width * oc] = px.reshape(height, width * oc)
    pix_off = 54 + (1024 if oc == 1 else 0)
    size = pix_off + stride * height
    head = struct.pack("<2sIIIIiiHHIIiiII", b"BM", size, 0, pix_off, 40, width, -height, 1,
                       8 if oc == 1 else 24, 0, 0, 0, 0, 256 if oc == 1 else 0, 0)
    pal = b""
    if oc == 1:
        pal = np.repeat(np.arange(256, dtype=np.uint8), 4).reshape(256, 4)
        pal[:, 3] = 0
        pal = pal.tobytes()
    return head + pal + rows.tobytes()


# ------------------------------------------------------------------- filter
def filter_rows(img, rows, rb, bpp, prior=None):
    """Adaptive PNG filter (src/gpu_filter.cu:183-309); returns rows*(rb+1) bytes."""
    img = np.ascontiguousarray(img, dtype=np.uint8).reshape(-1)
    assert img.size == rows * rb
    out = np.empty(rows * (rb + 1), np.uint8)
    pr = None if prior is None else np.ascontiguousarray(prior, dtype=np.uint8)
    lib().orc_filter_rows(_ptr(img), _ptr(pr) if pr is not None else None, rows, rb, bpp, _ptr(out))
    return out


def unfilter(filt, rows, rb, bpp):
    filt = np.ascontiguousarray(filt, dtype=np.uint8).reshape(-1)
    out = np.empty(rows * rb, np.uint8)
    if lib().orc_unfilter(_ptr(filt), rows, rb, bpp, _ptr(out)) != 0:
        raise ValueError("bad PNG filter type byte")
    return out


# --------------------------------------------------------------------- PNG
PNG_SIG = b"\x89PNG\r\n\x1a\n"


def parse_png(data):
    """Walk the chunks, verify every CRC with zlib.crc32, inflate the IDAT
    stream with zlib (which verifies the Adler-32 trailer) and unfilter.
    Returns (ihdr dict, pixel bytes, raw zlib stream, chunk list)."""
    data = bytes(data)
    if data[:8] != PNG_SIG:
        raise ValueError("bad PNG signature")
    pos, chunks, idat = 8, [], []
    ihdr = None
    while pos < len(data):
        (ln,) = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + ln]
        (crc,) = struct.unpack(">I", data[pos + 8 + ln:pos + 12 + ln])
        if zlib.crc32(typ + body) & 0xFFFFFFFF != crc:
            raise ValueError("CRC mismatch in %r chunk at %d" % (typ, pos))
        chunks.append((typ, ln))
        if typ == b"IHDR":
            w, h, depth, ctype, comp, flt, il = struct.unpack(">IIBBBBB", body)
            ihdr = dict(width=w, height=h, bit_depth=depth, color_type=ctype,
                        compression=comp, filter=flt, interlace=il)
        elif typ == b"IDAT":
            idat.append(body)
        pos += 12 + ln
        if typ == b"IEND":
            break
    if pos != len(data):
        raise ValueError("trailing bytes after IEND")
    stream = b"".join(idat)
    filt = zlib.decompress(stream)  # checks the zlib header and Adler-32
    ch = {0: 1, 2: 3, 4: 2, 6: 4}[ihdr["color_type"]]
    bpp = ch * ihdr["bit_depth"] // 8
    rb = ihdr["width"] * bpp
    if len(filt) != ihdr["height"] * (rb + 1):
        raise ValueError("inflated size %d != %d" % (len(filt), ihdr["height"] * (rb + 1)))
    pixels = unfilter(np.frombuffer(filt, np.uint8), ihdr["height"], rb, bpp)
    return ihdr, pixels, stream, chunks, np.frombuffer(filt, np.uint8)


# ------------------------------------------------------------ CPU pipeline
class PortEncoder:
    """CPU restatement of the reference's encode path (timed CPU baseline)."""

    def __init__(self, threads):
        self.threads = threads
        self.h = lib().port_encoder_create(threads)

    def close(self):
        if self.h:
            lib().port_encoder_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def encode(self, raw, width, height, channels, in_bytes, window_mode, params, level,
               strip_height, want_filtered=False):
        raw = np.ascontiguousarray(raw, dtype=np.uint8).reshape(-1)
        out_b = 1 if window_mode == 2 else in_bytes
        rb = width * channels * out_b
        cap = height * (rb + 1) * 2 + 65536
        out = np.empty(cap, np.uint8)
        filt = np.empty(height * (rb + 1), np.uint8) if want_filtered else None
        n = lib().port_encode_png(self.h, _ptr(raw), width, height, channels, in_bytes,
                                  window_mode, ctypes.byref(params) if params is not None else None,
                                  level, strip_height, _ptr(out), cap,
                                  _ptr(filt) if filt is not None else None)
        if n == 0:
            raise RuntimeError("port encoder output overflow")
        return (out[:n].tobytes(), filt) if want_filtered else out[:n].tobytes()

    def png_from_filtered(self, filt, width, height, rb, bit_depth, channels, level, strip_height):
        filt = np.ascontiguousarray(filt, dtype=np.uint8)
        cap = filt.size * 2 + 65536
        out = np.empty(cap, np.uint8)
        n = lib().port_png_from_filtered(self.h, _ptr(filt), width, height, rb, bit_depth, channels,
                                         level, strip_height, _ptr(out), cap)
        return out[:n].tobytes()


# ------------------------------------------------------- reference harness
def ref_available():
    return os.path.exists(os.path.join(HERE, "_ref", "libref_window.so"))


_ref_win = None
_ref_cpu = None


def ref_window_lib():
    global _ref_win
    if _ref_win is None:
        L = ctypes.CDLL(os.path.join(HERE, "_ref", "libref_window.so"))
        P = ctypes.POINTER(OrcParams)
        L.ref_window8.argtypes = [_u8p, _u8p, ctypes.c_int, P]
        L.ref_window8.restype = ctypes.c_int
        L.ref_try_apply_linear_window.argtypes = [_u8p, _u8p, ctypes.c_int, P]
        L.ref_try_apply_linear_window.restype = ctypes.c_int
        L.ref_build_dicom16_lut.argtypes = [_u8p, P, ctypes.c_int]
        _ref_win = L
    return _ref_win


def ref_bmp_runner():
    """Path of oracle/_ref/ref_bmp_runner (the reference's BMP export), or None."""
    path = os.path.join(HERE, "_ref", "ref_bmp_runner")
    return path if os.path.exists(path) else None


def ref_bmp_file(raw, width, height, channels, bits_per_sample, p=None, workdir=None):
    """BMP bytes the reference's own encode_source_to_bmp writes for an image
    (p: DicomPixelParams of a DICOM source, None for TIFF/RAW)."""
    import subprocess
    import tempfile
    runner = ref_bmp_runner()
    assert runner, "reference BMP runner not built"
    with tempfile.TemporaryDirectory(dir=workdir) as td:
        src, dst = os.path.join(td, "in.raw"), os.path.join(td, "out.bmp")
        np.ascontiguousarray(raw, dtype=np.uint8).tofile(src)
        q = p if p is not None else make_params()
        args = [runner, src, dst, str(width), str(height), str(channels), str(bits_per_sample),
                "1" if p is not None else "0", str(q.bits_allocated), str(q.bits_stored), str(q.high_bit),
                str(q.pixel_rep), str(q.apply_rescale), float(q.rescale_slope).hex(),
                float(q.rescale_intercept).hex(), str(q.apply_window), float(q.window_center).hex(),
                float(q.window_width).hex()]
        subprocess.run(args, check=True)
        with open(dst, "rb") as f:
            return f.read()


def ref_window8(raw_le, p):
    raw_le = np.ascontiguousarray(raw_le, dtype=np.uint8).reshape(-1)
    out = np.empty(raw_le.size // 2, np.uint8)
    path = ref_window_lib().ref_window8(_ptr(raw_le), _ptr(out), out.size, ctypes.byref(p))
    return out, path


def ref_build_lut(p):
    n = 1 << p.bits_stored
    lut = np.empty(n, np.uint8)
    ref_window_lib().ref_build_dicom16_lut(_ptr(lut), ctypes.byref(p), n)
    return lut


def ref_cpu_png_from_filtered(filt, width, height, rb, bit_depth, channels, level, strip_height,
                              threads, path):
    global _ref_cpu
    if _ref_cpu is None:
        L = ctypes.CDLL(os.path.join(HERE, "_ref", "libref_cpu.so"))
        L.ref_cpu_png_from_filtered.argtypes = [_u8p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_char_p]
        L.ref_cpu_png_from_filtered.restype = ctypes.c_int
        _ref_cpu = L
    filt = np.ascontiguousarray(filt, dtype=np.uint8)
    ok = _ref_cpu.ref_cpu_png_from_filtered(_ptr(filt), width, height, rb, bit_depth, channels, level,
                                            strip_height, threads, path.encode())
    if not ok:
        raise RuntimeError("reference PngWriter could not open %s" % path)
    with open(path, "rb") as f:
        return f.read()
