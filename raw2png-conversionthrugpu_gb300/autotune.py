"""Autotuner for the size-class table (r2p_tuning).

For each image-size class of the batched CT workload it times candidate
(DEFLATE block size, filter rows per work item, LZ77 hash-table bits) on a
planned batch of that class, replayed as a CUDA graph, keeps the fastest
candidate whose output is within 1% of the smallest (on the CT slices and
on 16-bit radial-gradient images of the class's size), then checks whole
tables on the mixed batch, and writes the table that Engine.set_tuning()
takes.  Runs on the
GPU; `python -m`-style entry: python raw2png-conversionthrugpu_gb300/autotune.py
[--out path.json].  The engine's built-in table (kDefaultTuning in
csrc/r2p_engine.cu) repeats the committed tuning_gb300.json;
tests/test_tuning_table.py fails when the two differ.
"""
import json
import os
import sys

import numpy as np

CLASSES = [(256, 256), (512, 512), (1024, 1024), (2048, 2500), (3072, 3072)]
CANDIDATES = [(bs, br, hb) for bs in (65520, 32752, 21760) for hb in (10, 9) for br in (0, 16, 32, 64, 128)]
DEFAULT_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_gb300.json")


def class_bounds():
    """Upper raw-byte bound of each class: halfway to the next class."""
    sizes = [w * h * 2 for w, h in CLASSES]
    return [(sizes[i] + sizes[i + 1]) // 2 for i in range(len(sizes) - 1)] + [2 ** 62]


def tune(r2p, W, reps=5, target_bytes=160 << 20, log=print):
    import torch
    eng = r2p.Engine(0)
    stream = r2p.Stream()
    table = []
    for (w, h), bound in zip(CLASSES, class_bounds()):
        k = max(4, min(256, target_bytes // (w * h * 2)))
        raws = [W.ct_phantom_torch(7000 + i, w, h) for i in range(k)]
        imgs = [W.image_ct8(w, h, 40.0 + 10 * i, 400.0 + 5 * i, level=1) for i in range(k)]
        caps = [r2p.png_bound(im) for im in imgs]
        outs = [torch.empty(c, dtype=torch.uint8, device="cuda") for c in caps]
        lens = torch.zeros(k, dtype=torch.int64, device="cuda")
        # a second data family for the compression guard: 16-bit radial
        # gradients with noise and flat rectangles (the C1 kind of image)
        g_raws = [torch.from_numpy(W.radial_rects(8000 + i, w, h).view(np.int16)).cuda() for i in range(2)]
        g_imgs = [W.image_ct16(w, h, 2048.0, 4096.0, level=1) for _ in range(2)]
        g_caps = [r2p.png_bound(im) for im in g_imgs]
        g_outs = [torch.empty(c, dtype=torch.uint8, device="cuda") for c in g_caps]
        g_lens = torch.zeros(2, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        results = []
        for cand in CANDIDATES:
            eng.set_tuning([(2 ** 62, cand[0], cand[1], cand[2])])
            b = eng.batch(imgs, [t.data_ptr() for t in raws], [t.data_ptr() for t in outs], caps, lens.data_ptr())
            b.launch_graph(stream)
            b.launch_graph(stream)
            e0, e1 = r2p.Event(), r2p.Event()
            times = []
            for _ in range(reps):
                e0.record(stream)
                b.launch_graph(stream)
                e1.record(stream)
                times.append(e0.elapsed_ms(e1))
            stream.sync()
            b.close()
            ms = sorted(times)[len(times) // 2]
            png_bytes = int(lens.sum().item())
            gb = eng.batch(g_imgs, [t.data_ptr() for t in g_raws], [t.data_ptr() for t in g_outs], g_caps,
                           g_lens.data_ptr())
            gb.launch(stream)
            stream.sync()
            gb.close()
            g_bytes = int(g_lens.sum().item())
            log("class %dx%d x%d  block %d band_rows %d hash_bits %d: %.3f ms (%.1f images/s), %d PNG bytes, "
                "%d on 16-bit gradients" % (w, h, k, cand[0], cand[1], cand[2], ms, k / ms * 1e3, png_bytes, g_bytes))
            results.append((ms, png_bytes, g_bytes, cand))
        # fastest candidate whose output is within 1% of the smallest on both data families
        s_ct = min(r[1] for r in results)
        s_g = min(r[2] for r in results)
        ms, png_bytes, g_bytes, cand = min((r for r in results if r[1] <= 1.01 * s_ct and r[2] <= 1.01 * s_g),
                                           key=lambda r: r[0])
        log("class %dx%d: block %d band_rows %d hash_bits %d (%.3f ms, %d / %d PNG bytes; smallest %d / %d)"
            % (w, h, cand[0], cand[1], cand[2], ms, png_bytes, g_bytes, s_ct, s_g))
        table.append((bound, cand[0], cand[1], cand[2]))
        del raws, outs, g_raws, g_outs
    eng.close()
    return table


def mixed_ms(r2p, W, eng, stream, table, n=1000, reps=5):
    """Graph-replay time of the mixed 1000-slice batch under a whole table:
    one LZ77 launch covers every class, so its shared memory (and CTAs per
    SM) follows the largest block any class picks."""
    import torch
    specs = W.mixed_batch_specs(n)
    raws = [W.ct_phantom_torch(sd, w, h) for (w, h, wc, ww, sd) in specs]
    imgs = [W.image_ct8(w, h, wc, ww, level=1) for (w, h, wc, ww, sd) in specs]
    eng.set_tuning(table)
    caps = [r2p.png_bound(im) for im in imgs]
    out = torch.empty(sum((c + 255) // 256 * 256 for c in caps), dtype=torch.uint8, device="cuda")
    offs, o = [], 0
    for c in caps:
        offs.append(o)
        o += (c + 255) // 256 * 256
    lens = torch.zeros(n, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    b = eng.batch(imgs, [t.data_ptr() for t in raws], [out.data_ptr() + x for x in offs], caps, lens.data_ptr())
    b.launch_graph(stream)
    b.launch_graph(stream)
    e0, e1 = r2p.Event(), r2p.Event()
    times = []
    for _ in range(reps):
        e0.record(stream)
        b.launch_graph(stream)
        e1.record(stream)
        times.append(e0.elapsed_ms(e1))
    stream.sync()
    b.close()
    del raws, out
    return sorted(times)[len(times) // 2]


def pick_table(r2p, W, per_class, log=print):
    """Per-class winners, or one block size for every class (keeping each
    class's band rows and hash bits), whichever runs the mixed batch fastest."""
    eng = r2p.Engine(0)
    stream = r2p.Stream()
    tables = {"per-class": per_class}
    for bs in (65520, 32752, 21760):
        tables["all %d" % bs] = [(c[0], bs, c[2], c[3]) for c in per_class]
    best = None
    for name, t in tables.items():
        ms = mixed_ms(r2p, W, eng, stream, t)
        log("mixed 1000-slice batch, %s table %s: %.3f ms" % (name, t, ms))
        if best is None or ms < best[0]:
            best = (ms, name, t)
    eng.close()
    log("chosen: %s (%.3f ms)" % (best[1], best[0]))
    return best[2]


def main():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import __graft_entry__ as g
    r2p = g.load_package()
    from raw2png_gb300 import workloads as W
    out = sys.argv[sys.argv.index("--out") + 1] if "--out" in sys.argv else DEFAULT_OUT
    table = pick_table(r2p, W, tune(r2p, W))
    with open(out, "w") as f:
        json.dump({"device": "GB300", "workload": "CT phantom slices, 8-bit window, LZ77 level 1",
                   "fields": ["max_raw_bytes", "block_size", "band_rows", "hash_bits"], "classes": table}, f,
                  indent=1)
    print("wrote", out, table)


if __name__ == "__main__":
    main()
