"""Benchmark: raw-pixel MB/s and images/s of the GB300 PNG encoder.

The default workload is the 3072x3072 uint16 image of the single-large-image
configuration (12 bits stored, DICOM PS3.3 window WC 2048 / WW 4096 to 16-bit
output, adaptive filter, LZ77 + fixed Huffman at level 1 in independent
65520-byte blocks, the configuration's "64 KB independent blocks").  Eight
distinct inputs (151 MB of raw pixels, more than the 129 MB L2) are encoded in
turn; a step is one pass over the eight (eight images).

  value     device-resident throughput: pixels and PNG in HBM, timed with CUDA
            events on the encode streams, max over ranks
  e2e       the same metric through r2p_encode_png_many with pinned host
            buffers: host->device pixels and device->host PNG inside the
            timed region
  roofline  dominant kernel: algorithmic bytes per launch / its mean duration
            (CUDA events around each stage in a single-stream pass)
  autotuned_blocks  the same images in the size-class table's block size
  reference_kernels the reference's own window + filter kernels (compiled for
            sm_103a from its sources, where the cubins were built) on the
            same image, beside this encoder's filter stage
  batched_c3 / served_c4  the batched and served configurations
  cpu_baseline  the oracle's CPU restatement of the reference path (window,
            filter, strip-parallel zlib level 1, PNG container) on this host

`--impl reference` times that CPU path alone (all host threads) on the same
workload and metric.  Multi-GPU runs (torchrun) are independent replicas:
each rank encodes its own images, no collective on the data path.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "raw-pixel MB/s"
UNIT = "MB/s"
IMAGES_PER_STEP = 8


def workload_desc(name):
    return {
        "c1": "single 3072x3072 uint16 image (12 bits stored), DICOM window WC 2048/WW 4096 to 16-bit, "
              "adaptive filter, LZ77 + fixed Huffman level 1 in 64 KB independent blocks",
        "c0": "single 512x512 uint16 CT phantom (12 bits stored), slope 1 / intercept -1024, WC 40/WW 400 to "
              "8-bit (Q15 path), adaptive filter, stored DEFLATE (level 0)",
        "c2": "single 6000x4000 RGB uint16 image, no window, adaptive filter, LZ77 + fixed Huffman level 1",
    }[name]


def make_inputs(W, name, nvar):
    if name == "c1":
        base = W.radial_rects(1, 3072, 3072)
        img = W.image_c1(level=1)
    elif name == "c0":
        base = W.ct_phantom(0)
        img = W.image_c0()
    else:
        base = W.rgb_sinusoids(2, 6000, 4000)
        img = W.image_c2(level=1)
    raws = [np.ascontiguousarray(np.roll(base, 97 * k, axis=1)) for k in range(nvar)]
    return img, raws


def cpu_params(O, img):
    return O.OrcParams.from_buffer_copy(bytes(img.dicom))


def window_mode_for_port(r2p, img):
    return {r2p.WINDOW_NONE: 0, r2p.WINDOW_DICOM16: 1, r2p.WINDOW_BATCH8: 2}[img.window_mode]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel, workload):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*%s\s+%s\s*=\s*([0-9]+)" % (re.escape(kernel), re.escape(workload)),
                  text)
    return int(m.group(1)) if m else None


def ncu_issue(kernel, workload):
    """Issue-active fraction of `kernel` from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.md")
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"issue_active_per_launch:\s*%s\s+%s\s*=\s*([0-9.]+)" % (re.escape(kernel), re.escape(workload)),
                  text)
    return float(m.group(1)) if m else None


TUNING_JSON = os.path.join(ROOT, "raw2png-conversionthrugpu_gb300", "tuning_gb300.json")


def load_tuning(eng):
    """Apply the committed autotuned size-class table, if present."""
    try:
        with open(TUNING_JSON) as f:
            t = json.load(f)
        eng.set_tuning([tuple(c) for c in t["classes"]])
        return "autotuned (%s)" % os.path.basename(TUNING_JSON)
    except (OSError, KeyError, ValueError):
        return "built-in"


def block_size_used(eng, img):
    """DEFLATE block size the engine's table gives this image: the class's
    size at level 1, 65520 at other levels, unless the image sets its own."""
    if img.block_size:
        return img.block_size
    if img.level != 1:
        return 65520
    classes = eng.get_tuning()
    for (max_raw, bs, _, _) in classes:
        if img.raw_bytes <= max_raw:
            return bs
    return classes[-1][1]


def measure_c3(r2p, W, eng, stream, n=1000, reps=3):
    """1000 mixed-size CT slices (8-bit window, LZ77 level 1): plain per-image
    calls vs one planned batch replayed as a CUDA graph.  Outputs of the two
    paths must be byte-identical."""
    import torch
    specs = W.mixed_batch_specs(n)
    raws = [W.ct_phantom_torch(sd, w, h) for (w, h, wc, ww, sd) in specs]
    imgs = [W.image_ct8(w, h, wc, ww, level=1) for (w, h, wc, ww, sd) in specs]
    caps = [r2p.png_bound(im) for im in imgs]
    offs, o = [], 0
    for c in caps:
        offs.append(o)
        o += (c + 255) // 256 * 256
    out_plain = torch.zeros(o, dtype=torch.uint8, device="cuda")
    out_batch = torch.zeros(o, dtype=torch.uint8, device="cuda")
    len_plain = torch.zeros(n, dtype=torch.int64, device="cuda")
    len_batch = torch.zeros(n, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    raw_bytes = sum(im.raw_bytes for im in imgs)
    e0, e1 = r2p.Event(), r2p.Event()

    def plain_pass():
        for i in range(n):
            eng.encode_png_device(imgs[i], raws[i].data_ptr(), out_plain.data_ptr() + offs[i], caps[i],
                                  len_plain.data_ptr() + 8 * i, stream)

    plain_pass()
    stream.sync()
    t_plain = []
    for _ in range(reps):
        e0.record(stream)
        plain_pass()
        e1.record(stream)
        t_plain.append(e0.elapsed_ms(e1))
    b = eng.batch(imgs, [t.data_ptr() for t in raws], [out_batch.data_ptr() + x for x in offs], caps,
                  len_batch.data_ptr())
    b.launch_graph(stream)
    b.launch_graph(stream)
    stream.sync()
    launches0 = r2p.launch_count()
    t_batch = []
    for _ in range(reps):
        e0.record(stream)
        b.launch_graph(stream)
        e1.record(stream)
        t_batch.append(e0.elapsed_ms(e1))
    stream.sync()
    graph_launches = (r2p.launch_count() - launches0) // reps
    same = bool(torch.equal(len_plain, len_batch)) and bool(torch.equal(out_plain, out_batch))
    png_bytes = int(len_batch.sum().item())
    dev_bytes = b.device_bytes
    # roofline of the batch's dominant kernel: the same work list launched
    # part after part on one stream with CUDA events between the stages
    eng.set_timing(True)
    b.launch(stream)
    stream.sync()
    st = eng.stage_times()
    eng.set_timing(False)
    b.close()
    filt_total = sum(im.filtered_bytes for im in imgs)
    stream_total = png_bytes - 63 * n
    alg = {"window_filter": raw_bytes + filt_total, "lz77_blocks": filt_total + stream_total,
           "stored_blocks": 2 * filt_total, "finish": 2 * stream_total, "prepare_window": 0, "unused": 0}
    dname, (dms, _) = max(st.items(), key=lambda kv: kv[1][0])
    peak, peak_kind = peaks()
    kname = r2p.filter_kernel(imgs[0]) if dname == "window_filter" else r2p.KERNELS[r2p.STAGES.index(dname)]
    roof = {"bound": "hbm", "kernel": kname, "achieved": round(alg[dname] / (dms / 1e3) / 1e9, 1), "peak": peak,
            "unit": "GB/s", "frac": round(alg[dname] / (dms / 1e3) / 1e9 / peak, 4), "peak_source": peak_kind,
            "algorithmic_bytes": alg[dname], "ms": round(dms, 3),
            "stage_ms": {k: round(v[0], 3) for k, v in st.items() if v[1]},
            "stage_gbs": {k: round(alg[k] / (v[0] / 1e3) / 1e9, 1) for k, v in st.items() if v[1] and alg[k]},
            "timing": "CUDA events between the stages of the batch's parts, launched one after another on one "
                      "stream (the graph runs the four parts side by side)"}
    mp, mb = statistics.median(t_plain), statistics.median(t_batch)
    res = {"images": n, "raw_bytes": raw_bytes, "png_bytes": png_bytes,
           "plain_images_per_s": round(n / mp * 1e3, 1), "plain_raw_MBps": round(raw_bytes / mp / 1e3, 1),
           "batched_images_per_s": round(n / mb * 1e3, 1), "batched_raw_MBps": round(raw_bytes / mb / 1e3, 1),
           "batched_vs_plain": round(mp / mb, 2), "plain_ms": round(mp, 3), "batched_ms": round(mb, 3),
           "kernels_per_graph": graph_launches, "batch_device_bytes": dev_bytes, "outputs_identical": same,
           "roofline": roof}
    del raws, out_plain, out_batch
    torch.cuda.empty_cache()
    return res


def measure_c4(r2p, W, n_pool=48, per_level=960, levels=(0.5, 0.8, 1.0), seed=4, threads=4, slots=8,
               batch_cap=0, batch_bytes=0):
    """Served request stream: Poisson arrivals at fractions of the measured
    saturation rate; p50/p99 latency (submit -> PNG in host memory) and images/s,
    next to the plain per-image path (r2p_encode_png, one image at a time)."""
    import random
    import threading
    specs = W.request_specs(n_pool, seed)
    import ctypes
    pool = []
    for (w, h, eight, wc, ww, sd) in specs:
        raw = W.ct_phantom_torch(sd, w, h).cpu().numpy().view(np.uint8).reshape(-1)
        img = W.image_ct8(w, h, wc, ww, level=1) if eight else W.image_ct16(w, h, wc, ww, level=1)
        pin = r2p.PinnedBuffer(img.raw_bytes)     # requests arrive in pinned host memory
        pin.array[:] = raw
        pool.append((img, pin))
    mean_raw = sum(im.raw_bytes for im, _ in pool) / len(pool)
    # plain per-image path on the same GPU: r2p_encode_png from the same pinned
    # buffers into a pinned PNG buffer, one image at a time
    eng = r2p.Engine(0)
    load_tuning(eng)
    out = r2p.PinnedBuffer(max(r2p.png_bound(im) for im, _ in pool))
    n = ctypes.c_size_t()

    def plain(img, pin):
        r2p.check(r2p.lib().r2p_encode_png(eng.h, ctypes.byref(img), pin.ptr, out.ptr, out.nbytes, ctypes.byref(n)))

    for img, pin in pool[:4]:
        plain(img, pin)
    t0 = time.perf_counter()
    for img, pin in pool:
        plain(img, pin)
    plain_ips = len(pool) / (time.perf_counter() - t0)
    eng.close()
    sv = r2p.Server(0, hbm_budget=40 << 30, host_pool_bytes=8 << 30, max_inflight_batches=slots,
                    max_batch_images=batch_cap, max_batch_bytes=batch_bytes)
    try:
        with open(TUNING_JSON) as f:
            sv.set_tuning([tuple(c) for c in json.load(f)["classes"]])
    except (OSError, KeyError, ValueError):
        pass

    def run(arrivals):
        """Submit request k at time arrivals[k] (seconds from start) from
        `threads` submitters; return (latencies ms, wall seconds)."""
        n = len(arrivals)
        tickets = [None] * n
        start = time.perf_counter() + 0.02

        def submitter(k):
            for i in range(k, n, threads):
                dt = start + arrivals[i] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                img, pin = pool[i % len(pool)]
                tickets[i] = sv.submit(img, pin, borrow=True)

        lat = [None] * n
        failed = []

        def waiter():
            # a client that takes each result as it completes (wait + release
            # in submission order), so finished PNGs do not pile up in the
            # server's pinned pool while the burst is still arriving
            for i in range(n):
                while tickets[i] is None:
                    time.sleep(0.0001)
                st, png_len, l, q = sv.wait(tickets[i], timeout_ms=120000, fetch=False)
                if st != r2p.OK or not png_len:
                    failed.append((tickets[i], st))
                lat[i] = l

        ths = [threading.Thread(target=submitter, args=(k,)) for k in range(threads)]
        wt = threading.Thread(target=waiter)
        for t in ths:
            t.start()
        wt.start()
        for t in ths:
            t.join()
        wt.join()
        if failed:
            raise RuntimeError(f"served requests failed: {failed[:4]}")
        wall = time.perf_counter() - start
        return lat, wall

    # saturation: everything arrives at once; median of five bursts of 2x the
    # per-level count (a burst lasts ~0.1 s, so single bursts vary by ~15 %)
    run([0.0] * 256)
    bursts = []
    for _ in range(5):
        sv.reset_stats()
        lat, wall = run([0.0] * (2 * per_level))
        bursts.append((2 * per_level / wall, sv.stats()))
    sats = [b[0] for b in bursts]
    sat, st = sorted(bursts, key=lambda b: b[0])[2]
    out = {"requests_per_level": per_level, "pool_images": len(pool), "mean_raw_bytes": int(mean_raw), "slots": slots,
           "max_batch_images": batch_cap or 512, "max_batch_bytes": batch_bytes or (96 << 20),
           "plain_images_per_s": round(plain_ips, 1), "saturation_images_per_s": round(sat, 1),
           "saturation_runs_images_per_s": [round(x, 1) for x in sats],
           "saturation_vs_plain": round(sat / plain_ips, 2), "mean_batch_images_at_saturation":
           round(st["mean_batch_images"], 1), "levels": []}
    rng = random.Random(seed)
    for f in levels:
        lam = f * sat
        t, arr = 0.0, []
        for _ in range(per_level):
            t += rng.expovariate(lam)
            arr.append(t)
        sv.reset_stats()
        lat, wall = run(arr)
        lat.sort()
        st = sv.stats()
        out["levels"].append({"load": f, "offered_images_per_s": round(lam, 1),
                              "achieved_images_per_s": round(per_level / wall, 1),
                              "p50_ms": round(lat[len(lat) // 2], 3),
                              "p99_ms": round(lat[min(len(lat) - 1, int(0.99 * (len(lat) - 1) + 0.5))], 3),
                              "mean_batch_images": round(st["mean_batch_images"], 2)})
    sv.close()
    return out


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, world, local, dist
    return 0, 1, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(O, r2p, img, raws, seconds=2.0, min_images=2):
    threads = os.cpu_count() or 1
    enc = O.PortEncoder(threads)
    mode = window_mode_for_port(r2p, img)
    p = cpu_params(O, img)
    strip = 256
    enc.encode(raws[0].view(np.uint8), img.width, img.height, img.channels, img.bytes_per_sample, mode, p,
               img.level, strip)   # warm the pool
    n, t0 = 0, time.perf_counter()
    while n < min_images or time.perf_counter() - t0 < seconds:
        enc.encode(raws[n % len(raws)].view(np.uint8), img.width, img.height, img.channels, img.bytes_per_sample,
                   mode, p, img.level, strip)
        n += 1
    dt = time.perf_counter() - t0
    enc.close()
    return {"value": round(n * img.raw_bytes / dt / 1e6, 2), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d images of the workload (%.1f s wall), strip height %d, zlib level %d, %d threads"
                      % (n, dt, strip, img.level, threads),
            "images_per_s": round(n / dt, 3)}


def run_reference(args):
    rank, world, local, dist = dist_setup()
    if rank != 0:
        return
    import __graft_entry__ as g
    r2p = g.load_package()
    from raw2png_gb300 import workloads as W
    from oracle import build_oracle, oracle as O
    build_oracle.build_oracle()
    img, raws = make_inputs(W, args.workload, 2)
    threads = os.cpu_count() or 1
    enc = O.PortEncoder(threads)
    mode = window_mode_for_port(r2p, img)
    p = cpu_params(O, img)
    row = img.width * img.channels * img.bytes_per_sample

    def enc_rows(k, rows):
        src = raws[k % 2].view(np.uint8).reshape(img.height, row)[:rows]
        enc.encode(src, img.width, rows, img.channels, img.bytes_per_sample, mode, p, img.level, 256)

    # a step is the whole image, or a band of its top rows when K whole images
    # would not finish within about 90 s on this host
    t0 = time.perf_counter()
    enc_rows(0, img.height)
    t_img = time.perf_counter() - t0
    rows = img.height
    if args.steps * t_img > 90.0:
        rows = max(64, min(img.height, int(img.height * 90.0 / (args.steps * t_img))))
    for i in range(args.warmup):
        enc_rows(i, rows)
    t0 = time.perf_counter()
    for i in range(args.steps):
        enc_rows(i, rows)
    dt = time.perf_counter() - t0
    enc.close()
    step_bytes = rows * row
    v = round(args.steps * step_bytes / dt / 1e6, 2)
    sample = ("%d steps of %d of the image's %d rows (%.1f MB raw each), strip height 256, zlib level %d, "
              "%d threads: CPU restatement of the reference's window/filter + its zlib strip pipeline"
              % (args.steps, rows, img.height, step_bytes / 1e6, img.level, threads))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt * 1e3 / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic", "config": {"workload": workload_desc(args.workload), "images_per_step": 1,
                                            "rows_per_step": rows},
            "images_per_s": round(args.steps * rows / img.height / dt, 3),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measure_dynamic(r2p, img, engines, streams, d_raw, nvar, steps):
    """The same workload at level 6 (dynamic Huffman blocks over a run-length
    parse), device-resident, steps dealt over the same engines and streams."""
    dimg = type(img).from_buffer_copy(img)
    dimg.level = 6
    S = len(engines)
    cap = r2p.png_bound(dimg)
    d_png = [[r2p.DeviceBuffer(cap) for _ in range(nvar)] for _ in range(S)]
    d_len = [r2p.DeviceBuffer(8 * nvar) for _ in range(S)]

    def step(i):
        s, k = i % S, i % nvar
        engines[s].encode_png_device(dimg, d_raw[k].ptr, d_png[s][k].ptr, cap, d_len[s].ptr + 8 * k, streams[s])

    for i in range(2 * S):
        step(i)
    for st in streams:
        st.sync()
    ev0, ev1 = r2p.Event(), r2p.Event()
    joins = [r2p.Event() for _ in range(S)]
    ev0.record(streams[0])
    for st in streams[1:]:
        st.wait(ev0)
    for i in range(steps):
        step(i)
    for s in range(1, S):
        joins[s].record(streams[s])
        streams[0].wait(joins[s])
    ev1.record(streams[0])
    streams[0].sync()
    ms = ev0.elapsed_ms(ev1)
    import zlib
    n0 = int(d_len[0].download(8 * nvar).view(np.uint64)[0])
    png = d_png[0][0].download(n0).tobytes()
    filt = zlib.decompress(png[41:len(png) - 16])
    assert len(filt) == dimg.filtered_bytes, "level-6 PNG does not inflate to the filtered size"
    return {"level": 6, "format": "dynamic Huffman blocks over a run-length parse (distance-1 matches)",
            "value": round(dimg.raw_bytes * steps / (ms / 1e3) / 1e6, 2), "unit": UNIT,
            "images_per_s": round(steps / (ms / 1e3), 2), "ms_per_step": round(ms / steps, 4), "steps": steps,
            "png_bytes": len(png), "zlib_level_6_stream": len(zlib.compress(filt, 6)),
            "ours_zlib_stream": len(png) - 57}


def timed_passes(r2p, engines, streams, img, d_raw, d_png, d_len, cap, steps):
    """`steps` passes over the rotated inputs (one image each), dealt
    round-robin to the engines and streams, joined on the first stream;
    device milliseconds between events around the whole region."""
    S, nvar = len(engines), len(d_raw)
    ev0, ev1 = r2p.Event(), r2p.Event()
    joins = [r2p.Event() for _ in range(S)]
    stream = streams[0]
    ev0.record(stream)
    for st in streams[1:]:
        st.wait(ev0)
    for i in range(steps * nvar):
        s, k = i % S, i % nvar
        engines[s].encode_png_device(img, d_raw[k].ptr, d_png[s][k].ptr, cap, d_len[s].ptr + 8 * k, streams[s])
    for s in range(1, S):
        joins[s].record(streams[s])
        stream.wait(joins[s])
    ev1.record(stream)
    stream.sync()
    return ev0.elapsed_ms(ev1)


def measure_reference_kernels(r2p, img, raw, strip_rows=1024, reps=10):
    """The reference's own window and filter kernels (src/gpu_filter.cu,
    compiled for sm_103a from the reference sources into oracle/_ref, with
    the reference's --use_fast_math) on the same image, launched with the
    reference's shape per strip of `strip_rows` rows (src/gpu_filter.cu:411-434; 1024
    rows is the modern path's default strip, include/pipeline.h:10-15):
    device microseconds per image.  A reported baseline, only where the
    cubins were built (they come from the reference tree)."""
    import ctypes
    ref = os.path.join(ROOT, "oracle", "_ref")
    cubin = os.path.join(ref, "gpu_filter_ref_fastmath.cubin")
    if not os.path.exists(cubin):
        return {"unavailable": "reference cubins not built here (the reference tree is absent)"}
    from oracle import build_oracle
    try:
        so = build_oracle.build_ref_gpu_runner()
        L = ctypes.CDLL(so)
    except (RuntimeError, OSError) as e:
        return {"unavailable": "reference kernel runner: %s" % str(e).splitlines()[0][:200]}
    if not hasattr(L, "rgr_time"):
        return {"unavailable": "runner without timing entry"}
    L.rgr_open.restype = ctypes.c_int
    L.rgr_open.argtypes = [ctypes.c_char_p]
    L.rgr_error.restype = ctypes.c_char_p
    L.rgr_time.restype = ctypes.c_int
    L.rgr_time.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                           ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_double)]
    h = L.rgr_open(cubin.encode())
    if h < 0:
        return {"unavailable": "cubin load: %s" % L.rgr_error().decode()}
    params = bytes(img.dicom)
    pbuf = ctypes.create_string_buffer(params, len(params))
    rbuf = np.ascontiguousarray(raw).view(np.uint8).reshape(-1)
    ms_pre, ms_filt = ctypes.c_double(), ctypes.c_double()
    # the reference windows only DICOM input (its kernel, 16-bit in and out)
    pp = ctypes.cast(pbuf, ctypes.c_void_p) if img.window_mode == r2p.WINDOW_DICOM16 else None
    rc = L.rgr_time(h, rbuf.ctypes.data, img.row_bytes, img.channels * img.out_bytes_per_sample, img.height, strip_rows,
                    pp, reps, ctypes.byref(ms_pre), ctypes.byref(ms_filt))
    if rc != 0:
        return {"unavailable": "reference kernels: %s" % L.rgr_error().decode()}
    tot = ms_pre.value + ms_filt.value
    return {"kernels": "dicom_preprocess_kernel + filter_select_kernel (reference release build, --use_fast_math)",
            "strip_rows": strip_rows, "window_us": round(ms_pre.value * 1e3, 2),
            "filter_us": round(ms_filt.value * 1e3, 2), "total_us": round(tot * 1e3, 2),
            "total_GBps": round((img.raw_bytes + img.filtered_bytes) / (tot / 1e3) / 1e9, 1),
            "timing": "CUDA events around each launch, summed over the image's strips, mean of %d passes" % reps}


def run_ours(args):
    rank, world, local, dist = dist_setup()
    import __graft_entry__ as g
    r2p = g.load_package()
    from raw2png_gb300 import workloads as W
    nvar = IMAGES_PER_STEP
    img, raws = make_inputs(W, args.workload, nvar)
    if args.workload == "c1":
        img.block_size = 65520     # the configuration's "64 KB independent blocks"
    # S engines on S streams, images dealt round-robin: images on different
    # streams overlap (one image alone leaves SMs idle in its LZ77 tail and
    # its per-image kernels)
    S = max(1, args.streams)
    engines = [r2p.Engine(local) for _ in range(S)]
    tuning = [load_tuning(e) for e in engines][0]
    eng = engines[0]
    streams = [r2p.Stream() for _ in range(S)]
    stream = streams[0]
    cap = r2p.png_bound(img)
    d_raw = [r2p.DeviceBuffer.from_array(r) for r in raws]
    d_png = [[r2p.DeviceBuffer(cap) for _ in range(nvar)] for _ in range(S)]
    d_len = [r2p.DeviceBuffer(8 * nvar) for _ in range(S)]

    def one(i, s):
        k = i % nvar
        engines[s].encode_png_device(img, d_raw[k].ptr, d_png[s][k].ptr, cap, d_len[s].ptr + 8 * k, streams[s])

    timed_passes(r2p, engines, streams, img, d_raw, d_png, d_len, cap, max(args.warmup, 1))
    # single-stream pass: per-stage CUDA-event times for the roofline and the
    # stage split (engine 0, one image at a time)
    eng.set_timing(True)
    for i in range(max(args.steps, nvar)):
        one(i, 0)
    stream.sync()
    stages = eng.stage_times()
    eng.set_timing(False)
    # timed region (device): `steps` passes over the eight inputs, all S streams
    clocks = ClockSampler(local)
    clocks.start()
    barrier(dist)
    stream.sync()
    launches0 = r2p.launch_count()
    ms = timed_passes(r2p, engines, streams, img, d_raw, d_png, d_len, cap, args.steps)
    barrier(dist)
    launches = r2p.launch_count() - launches0
    clk = clocks.stop()
    ms_max = max_over_ranks(dist, ms)
    images = args.steps * nvar
    value = img.raw_bytes * images * world / (ms_max / 1e3) / 1e6
    # output sanity (not timed): one PNG inflates to the right size
    lens = d_len[0].download(8 * nvar).view(np.uint64)
    png = d_png[0][0].download(int(lens[0])).tobytes()
    import zlib
    filt = zlib.decompress(png[41:len(png) - 16])      # IDAT data: zlib header .. Adler-32
    assert len(filt) == img.filtered_bytes, "benchmarked PNG does not inflate to the filtered size"
    comp_bytes = len(png)
    # compressed size beside zlib on the same filtered scanlines (not timed;
    # zlib-ng is not installed, the system zlib stands in)
    sizes = {"ours_zlib_stream": len(png) - 57, "filtered_bytes": len(filt)}
    for lv in (0, 1, 6):
        sizes["zlib_level_%d" % lv] = len(zlib.compress(filt, lv))
    sizes["zlib_version"] = zlib.ZLIB_RUNTIME_VERSION
    if img.level == 1 and sizes["ours_zlib_stream"] >= len(filt):
        sizes["note"] = ("fixed-Huffman LZ77 finds almost no repeats in this data: every level-1 block came out "
                         "smaller as a stored block; levels 2-9 (dynamic Huffman) compress it")
    # the autotuned block size (the size-class table's) on the same images
    tuned = None
    if img.block_size:
        timg = type(img).from_buffer_copy(img)
        timg.block_size = 0
        tcap = r2p.png_bound(timg)
        t_png = [[r2p.DeviceBuffer(tcap) for _ in range(nvar)] for _ in range(S)]
        timed_passes(r2p, engines, streams, timg, d_raw, t_png, d_len, tcap, 1)
        tms = timed_passes(r2p, engines, streams, timg, d_raw, t_png, d_len, tcap, args.steps)
        tl = d_len[0].download(8 * nvar).view(np.uint64)
        tuned = {"block_size": block_size_used(engines[0], timg), "value": round(img.raw_bytes * images / (tms / 1e3)
                                                                                / 1e6, 2),
                 "unit": UNIT, "ms_per_step": round(tms / args.steps, 4), "png_bytes": int(tl[0])}
        del t_png
    # e2e through the host entry point with pinned buffers: every image's
    # pixels go host->device and its PNG device->host inside the timed region
    import ctypes
    import threading
    L = r2p.lib()
    e2e_api = ""
    e2e_images = images
    if args.e2e_api == "many":
        # one host thread, r2p_encode_png_many over all images: up to 4 in
        # flight (helper engines)
        pins = [r2p.PinnedBuffer(img.raw_bytes) for _ in range(2)]
        for k in range(2):
            pins[k].array[:] = raws[k].view(np.uint8).reshape(-1)
        ring = [r2p.PinnedBuffer(cap) for _ in range(2 * r2p.MANY_SLOTS)]
        e2e_eng = r2p.Engine(local)
        load_tuning(e2e_eng)

        def many(count):
            sts, lens = e2e_eng.encode_png_many([img] * count, [pins[i % 2] for i in range(count)],
                                                [ring[i % len(ring)] for i in range(count)])
            assert all(st == r2p.OK for st in sts), sts[:8]
            return lens

        many(2 * r2p.MANY_SLOTS)
        barrier(dist)
        t0 = time.perf_counter()
        lens_e2e = many(e2e_images)
        t1 = time.perf_counter()
        barrier(dist)
        assert lens_e2e[0] == comp_bytes, "e2e PNG size differs from the device-resident run"
        e2e_eng.close()
        e2e_api = ("r2p_encode_png_many (pinned host buffers, up to %d images in flight), 1 host thread"
                   % r2p.MANY_SLOTS)
    T = max(1, args.e2e_threads)
    workers = []
    for t in range(T if args.e2e_api == "threads" else 0):
        we = r2p.Engine(local)
        load_tuning(we)
        pins = [r2p.PinnedBuffer(img.raw_bytes) for _ in range(2)]
        for k in range(2):
            pins[k].array[:] = raws[(2 * t + k) % nvar].view(np.uint8).reshape(-1)
        workers.append((we, pins, r2p.PinnedBuffer(cap)))

    def e2e_run(t, count):
        we, pins, pout = workers[t]
        n = ctypes.c_size_t()
        for i in range(count):
            r2p.check(L.r2p_encode_png(we.h, ctypes.byref(img), pins[i % 2].ptr, pout.ptr, cap, ctypes.byref(n)))

    if args.e2e_api == "threads":
        for t in range(T):
            e2e_run(t, 2)
        share = [e2e_images // T + (1 if t < e2e_images % T else 0) for t in range(T)]
        barrier(dist)
        t0 = time.perf_counter()
        ths = [threading.Thread(target=e2e_run, args=(t, share[t])) for t in range(T)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        t1 = time.perf_counter()
        barrier(dist)
        for we, _, _ in workers:
            we.close()
        e2e_api = "r2p_encode_png (pinned host buffers), %d worker thread(s), one engine each" % T
    e2e_s = max_over_ranks(dist, t1 - t0)
    e2e_value = img.raw_bytes * e2e_images * world / e2e_s / 1e6
    if rank != 0:
        return
    # roofline of the dominant kernel
    peak, peak_kind = peaks()
    dom = max(stages.items(), key=lambda kv: kv[1][0])
    dname, (dms, dl) = dom
    per_launch_ms = dms / max(dl, 1)
    stream_bytes = comp_bytes - 63
    alg = {"window_filter": img.raw_bytes + img.filtered_bytes,
           "lz77_blocks": img.filtered_bytes + stream_bytes,
           "stored_blocks": img.filtered_bytes + stream_bytes,
           "finish": 2 * stream_bytes,
           "prepare_window": 0, "unused": 0}
    achieved = alg[dname] / (per_launch_ms / 1e3) / 1e9
    kname = r2p.filter_kernel(img) if dname == "window_filter" else r2p.KERNELS[r2p.STAGES.index(dname)]
    stage_ms = {k: round(v[0] / max(v[1], 1), 5) for k, v in stages.items() if v[1]}
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": workload_desc(args.workload), "images_per_step": nvar,
                   "step": "one pass over %d distinct inputs (%.0f MB raw > 129 MB L2)"
                           % (nvar, nvar * img.raw_bytes / 1e6),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "streams_per_gpu": S},
        "images_per_s": round(images * world / (ms_max / 1e3), 2),
        "png_bytes": comp_bytes,
        "compressed_vs_zlib": sizes,
        "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": img.raw_bytes * nvar,
                "d2h_bytes_per_step": (comp_bytes + 8) * nvar,
                "images_per_s": round(e2e_images * world / e2e_s, 2),
                "api": e2e_api},
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": alg[dname], "ms_per_launch": round(per_launch_ms, 5),
                     "timing": "CUDA events around each launch, single-stream pass over the same images",
                     "traffic": ncu_traffic(kname, args.workload)},
        "stages_ms_per_image": stage_ms,
        "stages_GBps": {k: round(alg[k] / (v / 1e3) / 1e9, 1) for k, v in stage_ms.items() if alg.get(k)},
        "clocks": clk,
        "gpu_launches": launches,
    }
    issue = ncu_issue(kname, args.workload)
    if issue is not None:
        line["roofline"]["issue_active"] = issue
        line["roofline"]["issue_note"] = ("fraction of cycles the kernel's schedulers issued an instruction "
                                          "(ncu, profiles/ncu_traffic.md)")
    line["config"]["tuning"] = tuning
    line["config"]["block_size"] = block_size_used(engines[0], img)
    if tuned:
        line["autotuned_blocks"] = tuned
    if args.workload in ("c1", "c2"):
        line["dynamic_huffman"] = measure_dynamic(r2p, img, engines, streams, d_raw, nvar,
                                                  min(args.steps * nvar, 300))
        line["reference_kernels"] = measure_reference_kernels(r2p, img, raws[0])
        if "total_us" in line["reference_kernels"] and "window_filter" in stage_ms:
            line["reference_kernels"]["ours_window_filter_us"] = round(stage_ms["window_filter"] * 1e3, 2)
            line["reference_kernels"]["ours_kernel"] = r2p.filter_kernel(img)
    if not args.no_batched:
        line["batched_c3"] = measure_c3(r2p, W, eng, stream)
        line["served_c4"] = measure_c4(r2p, W, slots=args.server_slots)
    if world == 1 and not args.no_cpu_baseline:
        from oracle import build_oracle, oracle as O
        build_oracle.build_oracle()
        line["cpu_baseline"] = cpu_baseline(O, r2p, img, raws)
    print(json.dumps(line), flush=True)


def run_c3(args):
    """--workload c3: the batched mixed-size slice workload as the headline
    (--c3-images N: the first N slices of the same seeded set, e.g. to keep an
    ncu capture within a few GB of device memory)."""
    import __graft_entry__ as g
    r2p = g.load_package()
    from raw2png_gb300 import workloads as W
    eng = r2p.Engine(0)
    tuning = load_tuning(eng)
    stream = r2p.Stream()
    res = measure_c3(r2p, W, eng, stream, n=args.c3_images, reps=max(3, args.steps))
    print(json.dumps({"metric": "raw-pixel MB/s (batched)", "value": res["batched_raw_MBps"], "unit": UNIT,
                      "n_gpus": 1, "steps": max(3, args.steps), "warmup": 2, "ms_per_step": res["batched_ms"],
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
                      "data": "synthetic", "config": {"workload": "%d CT phantom slices, sides {256^2, 512^2, "
                                                                  "1024^2, 2048x2500, 3072^2}, 8-bit window, LZ77 "
                                                                  "level 1" % args.c3_images, "tuning": tuning},
                      "batched_c3": res}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c1", choices=["c1", "c0", "c2", "c3", "c4"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--e2e-threads", type=int, default=6)
    ap.add_argument("--e2e-api", default="many", choices=["many", "threads"])
    ap.add_argument("--streams", type=int, default=8)
    ap.add_argument("--server-slots", type=int, default=8)
    ap.add_argument("--c3-images", type=int, default=1000)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "c3":
        run_c3(args)
    elif args.workload == "c4":
        import __graft_entry__ as g
        r2p = g.load_package()
        from raw2png_gb300 import workloads as W
        print(json.dumps({"metric": "served images/s and p50/p99 latency",
                          "served_c4": measure_c4(r2p, W, slots=args.server_slots)}),
              flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
