"""Serving: continuous batching with pooled device memory and HBM-budget
admission (r2p_server_*).

Requests arrive from several threads while earlier batches are on the GPU;
each result must be byte-identical to encoding the same image alone, and
decode (oracle PNG reader) to the oracle's pixels.  Admission must keep the
device pool within its budget, over-budget requests are refused, and waits,
cancels and failures report a status instead of hanging.
"""
import threading

import numpy as np
import pytest

from test_gpu_png import decode_and_check

pytestmark = pytest.mark.gpu


def requests(r2p, W, n, seed, cap=640, levels=(1,)):
    out = []
    for i, (w, h, eight, wc, ww, sd) in enumerate(W.request_specs(n, seed)):
        w, h = min(w, cap), min(h, cap)
        raw = W.ct_phantom(sd, w, h)
        lv = levels[i % len(levels)]
        img = W.image_ct8(w, h, wc, ww, level=lv) if eight else W.image_ct16(w, h, wc, ww, level=lv)
        out.append((img, raw))
    return out


@pytest.mark.parametrize("levels", [(1,), (0, 1, 6, 9)])
def test_results_same_alone_and_in_the_mix(engine, O, r2p, W, levels):
    items = requests(r2p, W, 48, seed=11, cap=640 if levels == (1,) else 2048, levels=levels)
    tickets = [None] * len(items)
    with r2p.Server(0, hbm_budget=1 << 30, host_pool_bytes=256 << 20, max_inflight_batches=3) as sv:
        def client(k):
            # clients 0 and 2 copy their pixels in; 1 and 3 lend them (zero-copy)
            for i in range(k, len(items), 4):
                tickets[i] = sv.submit(*items[i], borrow=bool(k & 1))

        ths = [threading.Thread(target=client, args=(k,)) for k in range(4)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        results = [sv.wait(t) for t in tickets]
        st = sv.stats()
    assert st["completed"] == len(items) and st["failed"] == 0
    assert st["batches"] >= 1 and st["p99_ms"] >= st["p50_ms"] > 0
    for i, (img, raw) in enumerate(items):
        status, png, lat, q = results[i]
        assert status == r2p.OK and lat >= q >= 0
        assert png == engine.encode_png(img, raw), "result differs from the same image encoded alone"
        if i % 8 == 0:
            decode_and_check(O, r2p, img, raw, png)


def test_admission_keeps_within_budget(r2p, W):
    items = requests(r2p, W, 16, seed=12, cap=512)
    budget = 24 << 20
    with r2p.Server(0, hbm_budget=budget, host_pool_bytes=64 << 20, max_inflight_batches=2) as sv:
        ts = [sv.submit(img, raw) for img, raw in items]
        res = [sv.wait(t) for t in ts]
        st = sv.stats()
        assert all(r[0] == r2p.OK for r in res)
        assert st["device_bytes_peak"] <= budget
        # a request that can never fit the budget is refused at submit
        big = W.image_ct16(4096, 4096, 40.0, 400.0)
        with pytest.raises(r2p.R2PError) as ei:
            sv.submit(big, np.zeros(4096 * 4096, "<u2"))
        assert ei.value.status == r2p.EBUDGET


def test_cancel_wait_and_bad_requests(r2p, W):
    items = requests(r2p, W, 24, seed=13, cap=640)
    with r2p.Server(0, hbm_budget=64 << 20, host_pool_bytes=128 << 20, max_inflight_batches=1,
                    max_batch_images=2) as sv:
        ts = [sv.submit(img, raw) for img, raw in items]
        cancelled = [t for t in ts[12:] if sv.cancel(t) == r2p.OK]
        for t in ts:
            status, png, lat, q = sv.wait(t, timeout_ms=60000)
            if t in cancelled:
                assert status == r2p.ECANCELED and png is None
            else:
                assert status == r2p.OK and png is not None
        assert sv.stats()["canceled"] == len(cancelled)
        # malformed requests and unknown tickets are reported, not crashed on
        bad = W.image_ct8(64, 64, 40.0, 400.0)
        bad.channels = 2
        with pytest.raises(r2p.R2PError) as ei:
            sv.submit(bad, np.zeros(64 * 64 * 2, "<u2"))
        assert ei.value.status == r2p.EINVAL
        assert sv.wait(999999, timeout_ms=0)[0] == r2p.ENOTFOUND
        # a bounded wait on work still queued returns ETIMEOUT or the result
        t = sv.submit(*items[0])
        st = sv.wait(t, timeout_ms=0, release=False)[0]
        assert st in (r2p.ETIMEOUT, r2p.OK)
        assert sv.wait(t)[0] == r2p.OK
