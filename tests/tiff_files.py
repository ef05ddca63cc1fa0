"""Writes small baseline TIFF files (TIFF 6.0: 8-byte header, one IFD of
12-byte entries, uncompressed strips) for the TIFF reader and CLI tests."""
import struct

import numpy as np


def write_tiff(path, img, order="II", rows_per_strip=7, photometric=None, compression=1, tiled=False,
               planar=1):
    """img: (H, W) or (H, W, C) uint8/uint16 samples (values, not bytes)."""
    a = np.asarray(img)
    if a.ndim == 2:
        a = a[..., None]
    h, w, c = a.shape
    bits = 8 * a.dtype.itemsize
    e = "<" if order == "II" else ">"
    data = a.astype(a.dtype.newbyteorder(e)).tobytes()
    row = w * c * a.dtype.itemsize
    strips = [data[r * row:min(h, r + rows_per_strip) * row] for r in range(0, h, rows_per_strip)]
    photometric = (2 if c >= 3 else 1) if photometric is None else photometric
    entries = []
    extra = b""
    base = 8
    # layout: header | pixel strips | extra arrays | IFD
    pix = b"".join(strips)
    offs, o = [], base
    for st in strips:
        offs.append(o)
        o += len(st)
    extra_off = base + len(pix)

    def arr(vals, typ):
        nonlocal extra
        fmt = "H" if typ == 3 else "I"
        raw = struct.pack(e + fmt * len(vals), *vals)
        if len(raw) <= 4:
            return raw.ljust(4, b"\0")
        at = extra_off + len(extra)
        extra += raw + (b"\0" if len(raw) % 2 else b"")
        return struct.pack(e + "I", at)

    def ent(tag, typ, vals):
        entries.append(struct.pack(e + "HHI", tag, typ, len(vals)) + arr(vals, typ))

    ent(256, 4, [w])
    ent(257, 4, [h])
    ent(258, 3, [bits] * c)
    ent(259, 3, [compression])
    ent(262, 3, [photometric])
    if tiled:
        ent(322, 3, [16])
    ent(273, 4, offs)
    ent(277, 3, [c])
    ent(278, 4, [rows_per_strip])
    ent(279, 4, [len(st) for st in strips])
    ent(284, 3, [planar])
    ifd_off = extra_off + len(extra)
    ifd = struct.pack(e + "H", len(entries)) + b"".join(entries) + struct.pack(e + "I", 0)
    hdr = (b"II*\0" if order == "II" else b"MM\0*") + struct.pack(e + "I", ifd_off)
    with open(path, "wb") as f:
        f.write(hdr + pix + extra + ifd)


def expected_png_bytes(img, photometric=None):
    """Samples as the reader delivers them: big-endian, MINISWHITE inverted."""
    a = np.asarray(img)
    b = a.astype(a.dtype.newbyteorder(">")).tobytes()
    out = np.frombuffer(b, np.uint8).copy()
    if photometric == 0:
        out ^= 0xFF
    return out
