"""Write tests/golden/bmp_ref.npz: BMP files written by the reference's own
BMP export (encode_source_to_bmp, src/pipeline.cpp:1944-2004 and
src/bmp_writer.cpp, built by oracle/build_oracle.py into oracle/_ref) for
seeded synthetic images, with their raw pixels and parameters.

Run where the reference tree is present:
    python tests/golden/gen_bmp_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build_oracle, oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bmp_ref.npz")


def p16(bits_stored=12, high_bit=None, pixel_rep=0, slope=None, intercept=None, wc=None, ww=None, ba=16):
    return oracle.make_params(ba, bits_stored, high_bit, pixel_rep, slope, intercept, wc, ww)


def params_dict(p):
    return {k: getattr(p, k) for k, _ in oracle.OrcParams._fields_}


def main():
    build_oracle.build_oracle()
    assert build_oracle.build_ref(), "reference sources not found"
    rng = np.random.default_rng(20261203)
    cases = []

    def le16(vals):
        return np.asarray(vals, dtype="<u2").tobytes()

    def add(name, raw, w, h, ch, bps, mode, p=None):
        """mode: dicom | be | batch8 (the BMP source the reference sees)."""
        raw = np.frombuffer(raw, np.uint8).copy()
        if mode == "batch8":
            # the folder batch converts 16->8 on the CPU first, then writes an
            # 8-bit gray source (src/batch_processor.cpp:389-422)
            px8, _ = oracle.ref_window8(raw, p)
            bmp = oracle.ref_bmp_file(px8, w, h, 1, 8, None)
        else:
            bmp = oracle.ref_bmp_file(raw, w, h, ch, 8 * bps, p if mode == "dicom" else None)
        meta = {"name": name, "width": w, "height": h, "channels": ch, "bytes_per_sample": bps, "mode": mode,
                "params": params_dict(p) if p is not None else None}
        cases.append((meta, raw, np.frombuffer(bmp, np.uint8).copy()))

    # 16-bit grayscale DICOM through the BMP path's own window formula
    ramp = np.arange(4096, dtype=np.uint16)
    # (2000, 3000) is a window where dividing by the range and multiplying by
    # its reciprocal (the batch table) round differently at two stored values
    for wc, ww in ((2048.0, 4096.0), (40.0, 400.0), (1000.5, 1.0), (3000.0, 7.25), (-500.0, 1500.0), (2000.0, 3000.0)):
        add("ramp12 wc=%g ww=%g" % (wc, ww), le16(ramp), 64, 64, 1, 2, "dicom", p16(12, wc=wc, ww=ww))
    add("ramp12 no window", le16(ramp), 64, 64, 1, 2, "dicom", p16(12))
    add("ramp12 signed no window", le16(ramp), 64, 64, 1, 2, "dicom", p16(12, pixel_rep=1))
    add("ramp12 signed rescale window", le16(ramp), 64, 64, 1, 2, "dicom",
        p16(12, pixel_rep=1, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0))
    add("ramp16 signed wide", le16(np.arange(0, 65536, 16, dtype=np.uint32)), 64, 64, 1, 2, "dicom",
        p16(16, pixel_rep=1, wc=0.0, ww=60000.0))
    add("ramp16 rescale 0.5", le16(np.arange(0, 65536, 16, dtype=np.uint32)), 64, 64, 1, 2, "dicom",
        p16(16, slope=0.5, intercept=-100.0, wc=12000.0, ww=20000.0))
    left = (rng.integers(0, 4096, 37 * 23) << 4).astype(np.uint16)            # high_bit 15: shift 4
    add("left-aligned 12-in-16", le16(left), 37, 23, 1, 2, "dicom", p16(12, high_bit=15, wc=2048.0, ww=4096.0))
    ct = rng.integers(0, 4096, 31 * 17).astype(np.uint16)
    add("ct odd width", le16(ct), 31, 17, 1, 2, "dicom", p16(12, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0))
    # 8-bit grayscale and 16-bit colour DICOM: no window in the reference's BMP path
    add("dicom 8-bit", rng.integers(0, 256, 29 * 11, dtype=np.uint8).tobytes(), 29, 11, 1, 1, "dicom",
        p16(8, wc=100.0, ww=50.0, ba=8))
    add("dicom rgb16", le16(rng.integers(0, 65536, 13 * 7 * 3)), 13, 7, 3, 2, "dicom", p16(16))
    # TIFF/RAW-like sources (big-endian 16-bit, or 8-bit)
    add("be16 gray", rng.integers(0, 256, 33 * 9 * 2, dtype=np.uint8).tobytes(), 33, 9, 1, 2, "be")
    add("be16 rgb", rng.integers(0, 256, 13 * 6 * 6, dtype=np.uint8).tobytes(), 13, 6, 3, 2, "be")
    add("be16 rgba", rng.integers(0, 256, 10 * 5 * 8, dtype=np.uint8).tobytes(), 10, 5, 4, 2, "be")
    add("u8 gray", rng.integers(0, 256, 19 * 7, dtype=np.uint8).tobytes(), 19, 7, 1, 1, "be")
    add("u8 rgb", rng.integers(0, 256, 10 * 9 * 3, dtype=np.uint8).tobytes(), 10, 9, 3, 1, "be")
    # folder batch: the 16->8 rule (Q15 and table paths), then an 8-bit gray BMP
    add("batch8 q15", le16(ct), 31, 17, 1, 2, "batch8", p16(12, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0))
    add("batch8 lut", le16(ct), 31, 17, 1, 2, "batch8", p16(12, slope=1.0, intercept=-1024.0, wc=40.0, ww=100.0))

    arrays = {"meta": np.array(json.dumps([m for m, _, _ in cases]))}
    for i, (_, raw, bmp) in enumerate(cases):
        arrays["raw_%d" % i] = raw
        arrays["bmp_%d" % i] = bmp
    np.savez_compressed(OUT, **arrays)
    print("wrote", OUT, len(cases), "cases")


if __name__ == "__main__":
    main()
