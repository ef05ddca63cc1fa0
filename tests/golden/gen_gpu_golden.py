"""Records golden vectors from the reference's own GPU kernels.

Runs dicom_preprocess_kernel and filter_select_kernel of the reference's
src/gpu_filter.cu -- compiled from the reference sources into
oracle/_ref/gpu_filter_ref_{ieee,fastmath}.cubin by oracle/build_oracle.py
(ieee: -prec-div=true -fmad=false; fastmath: --use_fast_math, the
reference's own build flag, CMakeLists.txt:190) -- through
oracle/ref_gpu_runner.cpp on a GPU, and writes tests/golden/gpu_filter_ref.npz:

  a2_<k>_params / a2_<k>_ieee   every stored value of one parameter set (the
        input is every 16-bit value 0..65535 little-endian, or every byte
        0..255 for 8-bit sets) through the window kernel (ieee build), and
  a2_<k>_fm_idx / a2_<k>_fm_val              where the fast-math build differs;
  flt_<k>_in / _prior / _params / _meta / _ieee / _fm / _pre_ieee / _pre_fm
        seeded strips through window (if params) + filter, both builds.

Needs a GPU and the cubins (built where the reference tree is present):
    python tests/golden/gen_gpu_golden.py [--out PATH]
"""
import argparse
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import build_oracle, oracle as O  # noqa: E402

# (bits_allocated, bits_stored, high_bit, pixel_rep, slope, intercept, wc, ww)
A2_SETS = [
    (16, 12, 11, 0, 1.0, -1024.0, 40.0, 400.0),      # CT, the 512x512 phantom's window
    (16, 12, 11, 0, None, None, 2048.0, 4096.0),     # no rescale, full-range window
    (16, 16, 15, 1, 1.5, -300.0, 100.0, 900.0),      # signed 16-bit, rescale
    (16, 12, 15, 0, None, None, 500.0, 1000.0),      # left-aligned: shift 4
    (16, 12, 11, 1, 1.0, -1024.0, None, None),       # signed 12-bit, rescale only
    (16, 16, 15, 0, None, None, None, None),         # identity (byte swap only)
    (16, 12, 11, 0, 0.5, 10.0, 7.5, 2.0),            # narrow, fractional window
    (16, 10, 9, 0, 2.0, -2048.0, -600.0, 80.0),      # 10 bits, negative centre
    (8, 8, 7, 0, None, None, 128.0, 200.0),          # 8-bit window (max 255)
    (8, 8, 7, 1, None, None, 0.0, 50.0),             # signed 8-bit
    (8, 6, 5, 0, 3.0, 5.0, 20.0, 30.0),              # 6 bits stored, rescale
]


def params_of(t):
    ba, bs, hb, pr, m, b, wc, ww = t
    return O.make_params(ba, bs, hb, pr, slope=m, intercept=b, wc=wc, ww=ww)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(ROOT, "tests", "golden", "gpu_filter_ref.npz"))
    args = ap.parse_args()
    lib = ctypes.CDLL(build_oracle.build_ref_gpu_runner())
    lib.rgr_open.restype = ctypes.c_int
    lib.rgr_error.restype = ctypes.c_char_p
    lib.rgr_run.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    ref = os.path.join(ROOT, "oracle", "_ref")
    h = {}
    for tag in ("ieee", "fastmath"):
        h[tag] = lib.rgr_open(os.path.join(ref, "gpu_filter_ref_%s.cubin" % tag).encode())
        if h[tag] < 0:
            raise SystemExit("cannot load %s cubin: %s" % (tag, lib.rgr_error().decode()))

    def run(tag, inp, prior, wb, bpp, rows, p):
        inp = np.ascontiguousarray(inp, np.uint8)
        out = np.zeros(rows * (wb + 1), np.uint8)
        pre = np.zeros(rows * wb, np.uint8)
        pb = (ctypes.c_ubyte * 40).from_buffer_copy(bytes(p)) if p is not None else None
        pr = np.ascontiguousarray(prior, np.uint8) if prior is not None else None
        rc = lib.rgr_run(h[tag], inp.ctypes.data, pr.ctypes.data if pr is not None else None, wb, bpp, rows,
                         ctypes.cast(pb, ctypes.c_void_p) if pb is not None else None, out.ctypes.data,
                         pre.ctypes.data)
        if rc:
            raise SystemExit("reference kernel run failed: %s" % lib.rgr_error().decode())
        return out, pre

    res = {}
    for k, t in enumerate(A2_SETS):
        p = params_of(t)
        if t[0] == 16:
            raw = np.arange(65536, dtype="<u2").view(np.uint8)
            wb, bpp = raw.size, 2
        else:
            raw = np.arange(256, dtype=np.uint8)
            wb, bpp = raw.size, 1
        _, pre_i = run("ieee", raw, None, wb, bpp, 1, p)
        _, pre_f = run("fastmath", raw, None, wb, bpp, 1, p)
        diff = np.nonzero(pre_i != pre_f)[0]
        res["a2_%d_params" % k] = np.frombuffer(bytes(p), np.uint8)
        res["a2_%d_ieee" % k] = pre_i
        res["a2_%d_fm_idx" % k] = diff.astype(np.int32)
        res["a2_%d_fm_val" % k] = pre_f[diff]
        print("a2 set %d: %d bytes differ between the ieee and fast-math builds" % (k, diff.size))

    rng = np.random.default_rng(2024)
    cases = []
    for bpp, wpx, rows in ((1, 37, 9), (2, 33, 7), (3, 29, 6), (4, 25, 5), (6, 21, 5), (8, 17, 4)):
        cases.append((bpp, wpx, rows, None, bool(rows % 2)))
    cases += [(2, 40, 8, 0, False), (2, 41, 6, 2, True), (1, 45, 5, 8, False), (2, 31, 6, 1, True),
              (2, 64, 5, 6, False), (1, 50, 4, 10, True)]
    for k, (bpp, wpx, rows, pset, with_prior) in enumerate(cases):
        wb = wpx * bpp
        # half smooth ramps (so every filter type wins somewhere), half noise
        x = np.arange(rows * wb) % 251
        noise = rng.integers(0, 256, size=rows * wb)
        inp = np.where(rng.random(rows * wb) < 0.5, (x * 7 + (np.arange(rows * wb) // wb) * 3) % 256, noise)
        inp = inp.astype(np.uint8)
        p = params_of(A2_SETS[pset]) if pset is not None else None
        if p is not None and A2_SETS[pset][0] == 16 and A2_SETS[pset][1] < 16:
            # keep stored values in range for half the samples
            v = inp.view("<u2").copy()
            v[::2] &= (1 << A2_SETS[pset][1]) - 1
            inp = v.view(np.uint8)
        prior = rng.integers(0, 256, size=wb).astype(np.uint8) if with_prior else None
        out_i, pre_i = run("ieee", inp, prior, wb, bpp, rows, p)
        out_f, pre_f = run("fastmath", inp, prior, wb, bpp, rows, p)
        res["flt_%d_in" % k] = inp
        res["flt_%d_prior" % k] = prior if prior is not None else np.zeros(0, np.uint8)
        res["flt_%d_params" % k] = np.frombuffer(bytes(p), np.uint8) if p is not None else np.zeros(0, np.uint8)
        res["flt_%d_meta" % k] = np.array([wpx, rows, bpp], np.int32)
        res["flt_%d_ieee" % k] = out_i
        res["flt_%d_fm" % k] = out_f
        res["flt_%d_pre_ieee" % k] = pre_i
        res["flt_%d_pre_fm" % k] = pre_f
    res["n_a2"] = np.array([len(A2_SETS)])
    res["n_flt"] = np.array([len(cases)])
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    np.savez_compressed(args.out, **res)
    print("wrote", args.out, os.path.getsize(args.out), "bytes")


if __name__ == "__main__":
    main()
