"""Generate golden vectors from the reference's own code (run where the
reference tree is present; the outputs are committed next to this script).

  window8_ref.npz  16->8-bit windowing by the reference's own
                   try_apply_linear_window / build_dicom16_lut /
                   apply_dicom16_lut (src/batch_processor.cpp:100-266) with its
                   dispatch (:397-409), for 64 parameter sets over a spread of
                   raw values, plus the 512x512 CT phantom.
  cpu_png_ref.json sha256 and size of PNGs written by the reference's own
                   deflate_strip + PngWriter (src/parallel_deflate.cpp,
                   src/png_writer.cpp) for fixed filtered inputs, so the CPU
                   port can be checked byte for byte.

Usage: python tests/golden/gen_golden.py   (needs oracle/_ref built by
oracle/build_oracle.py)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle, oracle as O  # noqa: E402
import __graft_entry__ as g  # noqa: E402


def param_sets():
    rng = np.random.default_rng(20240601)
    sets = [dict(bs=12, hb=11, pr=0, slope=1.0, intercept=-1024.0, wc=40.0, ww=400.0)]
    while len(sets) < 64:
        bs = int(rng.choice([8, 10, 12, 14, 16]))
        kw = dict(bs=bs, hb=bs - 1 if rng.random() < 0.75 else 15, pr=int(rng.random() < 0.3))
        if rng.random() < 0.7:
            kw["slope"] = float(np.float32(rng.choice([1.0, 0.5, 2.0, rng.uniform(0.1, 3.0)])))
            kw["intercept"] = float(np.float32(rng.choice([0.0, -1024.0, rng.uniform(-3000, 3000)])))
        if rng.random() < 0.85:
            kw["wc"] = float(np.float32(rng.uniform(-1000, 3000)))
            kw["ww"] = float(np.float32(rng.choice([rng.uniform(1, 300), rng.uniform(80, 1600),
                                                    rng.uniform(1000, 70000)])))
        sets.append(kw)
    return sets


def to_params(k):
    return O.make_params(16, k["bs"], k["hb"], k["pr"], slope=k.get("slope"), intercept=k.get("intercept"),
                         wc=k.get("wc"), ww=k.get("ww"))


def main():
    build_oracle.build_oracle()
    assert build_oracle.build_ref(), "reference tree not found"
    raw_vals = np.unique(np.concatenate([np.arange(0, 65536, 7), np.arange(0, 4200), [65535, 32767, 32768]]))
    raw_vals = raw_vals.astype("<u2")
    sets = param_sets()
    outs, paths, fields = [], [], []
    for k in sets:
        p = to_params(k)
        out, path = O.ref_window8(raw_vals.view(np.uint8), p)
        outs.append(out)
        paths.append(path)
        fields.append([p.bits_allocated, p.bits_stored, p.high_bit, p.pixel_rep, p.apply_rescale,
                       p.rescale_slope, p.rescale_intercept, p.apply_window, p.window_center, p.window_width])
    pkg = g.load_package()
    from raw2png_gb300 import workloads as W
    c0 = W.ct_phantom(0)
    c0_out, c0_path = O.ref_window8(c0.view(np.uint8), to_params(sets[0]))
    np.savez_compressed(os.path.join(HERE, "window8_ref.npz"), raw=raw_vals, params=np.array(fields, np.float64),
                        out=np.stack(outs), path=np.array(paths, np.int32), c0_raw=c0, c0_out=c0_out,
                        c0_path=np.int32(c0_path))
    # reference CPU codec on fixed filtered inputs
    cases = []
    filt_c0 = O.filter_rows(c0_out, 512, 512, 1)
    rng = np.random.default_rng(5)
    small = (rng.integers(0, 40, size=200 * 333) + np.arange(200 * 333) // 97 % 7).astype(np.uint8)
    filt_small = O.filter_rows(small, 200, 333, 1)
    for name, filt, w, h, rb, level, sh, thr in (("c0_level0_strip128_t8", filt_c0, 512, 512, 512, 0, 128, 8),
                                                 ("c0_level1_strip128_t8", filt_c0, 512, 512, 512, 1, 128, 8),
                                                 ("small_level6_strip16_t3", filt_small, 333, 200, 333, 6, 16, 3)):
        path = "/tmp/r2p_golden_%s.png" % name
        png = O.ref_cpu_png_from_filtered(filt, w, h, rb, 8, 1, level, sh, thr, path)
        cases.append(dict(name=name, width=w, height=h, level=level, strip_height=sh, threads=thr,
                          size=len(png), sha256=hashlib.sha256(png).hexdigest()))
    with open(os.path.join(HERE, "cpu_png_ref.json"), "w") as f:
        json.dump(dict(zlib="1.3", cases=cases), f, indent=1)
    print("wrote", len(sets), "window parameter sets and", len(cases), "PNG cases")


if __name__ == "__main__":
    main()
