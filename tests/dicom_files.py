"""Writes small DICOM Part-10 files for the reader and CLI tests.

Encodings follow DICOM PS3.10 section 7 (128-byte preamble, "DICM", file
meta group 0002 in Explicit VR Little Endian) and PS3.5 section 7.1 (data
elements in Explicit or Implicit VR Little Endian; OB/OW/SQ/UN/UT with two
reserved bytes and a 32-bit length).  Values are padded to even length.
"""
import struct

import numpy as np

IMPLICIT_LE = "1.2.840.10008.1.2"
EXPLICIT_LE = "1.2.840.10008.1.2.1"
JPEG_LOSSLESS = "1.2.840.10008.1.2.4.70"
LONG_VRS = {"OB", "OD", "OF", "OL", "OV", "OW", "SQ", "UC", "UR", "UT", "UN"}


def _pad(v, vr):
    if isinstance(v, str):
        v = v.encode("ascii")
    if len(v) % 2:
        v += b"\0" if vr in ("UI", "OB") else b" "
    return v


def element(group, elem, vr, value, explicit=True):
    value = _pad(value, vr)
    tag = struct.pack("<HH", group, elem)
    if not explicit:
        return tag + struct.pack("<I", len(value)) + value
    if vr in LONG_VRS:
        return tag + vr.encode() + b"\0\0" + struct.pack("<I", len(value)) + value
    return tag + vr.encode() + struct.pack("<H", len(value)) + value


def sequence_undefined(group, elem, items, explicit=True):
    """SQ of undefined length whose items (lists of element bytes) are of
    undefined length too, closed by item and sequence delimiters."""
    tag = struct.pack("<HH", group, elem)
    head = tag + (b"SQ\0\0" if explicit else b"") + struct.pack("<I", 0xFFFFFFFF)
    body = b""
    for it in items:
        body += struct.pack("<HHI", 0xFFFE, 0xE000, 0xFFFFFFFF) + b"".join(it)
        body += struct.pack("<HHI", 0xFFFE, 0xE00D, 0)
    return head + body + struct.pack("<HHI", 0xFFFE, 0xE0DD, 0)


def us(v):
    return struct.pack("<H", v)


def write_dicom(path, frames, bits_allocated=16, bits_stored=12, high_bit=None, pixel_rep=0, slope=None,
                intercept=None, wc=None, ww=None, transfer_syntax=EXPLICIT_LE, preamble=True, nested=True,
                photometric=None, number_of_frames=None):
    """frames: (H, W) one grayscale frame, (F, H, W) grayscale frames or (F, H, W, C), uint8/uint16 samples.
    wc/ww/slope/intercept: numbers or DS strings (e.g. "40\\\\400"); None leaves the tag out."""
    a = np.asarray(frames)
    if a.ndim == 2:          # one grayscale frame
        a = a[None]
    if a.ndim == 3:          # grayscale frames
        a = a[..., None]
    nf, h, w, c = a.shape
    explicit = transfer_syntax != IMPLICIT_LE
    sop = "1.2.840.10008.5.1.4.1.1.2"
    meta = (element(0x0002, 0x0001, "OB", b"\x00\x01") + element(0x0002, 0x0002, "UI", sop) +
            element(0x0002, 0x0003, "UI", "1.2.3.4.5.6.7") + element(0x0002, 0x0010, "UI", transfer_syntax) +
            element(0x0002, 0x0012, "UI", "1.2.3.4.99"))
    meta = element(0x0002, 0x0000, "UL", struct.pack("<I", len(meta))) + meta
    E = lambda g, e, vr, v: element(g, e, vr, v, explicit)
    ds = E(0x0008, 0x0016, "UI", sop) + E(0x0008, 0x0060, "CS", "CT")
    if nested:
        ds += sequence_undefined(0x0008, 0x1140, [[E(0x0008, 0x1150, "UI", sop), E(0x0008, 0x1155, "UI", "1.2.3")],
                                                  [sequence_undefined(0x0040, 0xA730, [[E(0x0040, 0xA040, "CS",
                                                                                          "TEXT")]], explicit)]],
                                  explicit)
    ds += E(0x0028, 0x0002, "US", us(c))
    ds += E(0x0028, 0x0004, "CS", photometric or ("MONOCHROME2" if c == 1 else "RGB"))
    if number_of_frames is not None or nf > 1:
        ds += E(0x0028, 0x0008, "IS", str(number_of_frames if number_of_frames is not None else nf))
    ds += E(0x0028, 0x0010, "US", us(h)) + E(0x0028, 0x0011, "US", us(w))
    ds += E(0x0028, 0x0100, "US", us(bits_allocated)) + E(0x0028, 0x0101, "US", us(bits_stored))
    if high_bit is not None:
        ds += E(0x0028, 0x0102, "US", us(high_bit))
    ds += E(0x0028, 0x0103, "US", us(pixel_rep))
    for tag, v in ((0x1050, wc), (0x1051, ww), (0x1052, intercept), (0x1053, slope)):
        if v is not None:
            ds += E(0x0028, tag, "DS", v if isinstance(v, str) else ("%.6g" % v))
    dt = "<u2" if bits_allocated == 16 else "u1"
    px = np.ascontiguousarray(a.astype(dt)).tobytes()
    ds += E(0x7FE0, 0x0010, "OW" if bits_allocated == 16 else "OB", px)
    with open(path, "wb") as f:
        if preamble:
            f.write(b"\0" * 128 + b"DICM" + meta)
        f.write(ds)
    return a
