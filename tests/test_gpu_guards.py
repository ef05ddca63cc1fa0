"""Guard bytes around every device output, a bounded device wait made to run
out, and an engine held to its HBM budget.

Each output buffer sits between 256-byte guard zones filled with a canary; a
kernel may write only the bytes it reports (the PNG / stream / file length,
the exact filtered size), so everything else must still hold the canary.
Device inputs are held in variables until the outputs are read back: a
temporary buffer would be freed before the kernels that read it run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CANARY = 0xA5
PAD = 256


class Guarded:
    def __init__(self, r2p, nbytes):
        self.n = int(nbytes)
        self.buf = r2p.DeviceBuffer(self.n + 2 * PAD)
        self.buf.memset(CANARY)
        self.ptr = self.buf.ptr + PAD

    def check(self, written):
        """Bytes [0, written) may change; the rest and both guards may not."""
        d = self.buf.download(self.n + 2 * PAD)
        assert (d[:PAD] == CANARY).all(), "write before the buffer"
        assert (d[PAD + written:] == CANARY).all(), "write past the reported length"
        return d[PAD:PAD + written].tobytes()


@pytest.mark.parametrize("level", [0, 1, 6])
@pytest.mark.parametrize("w,h,ch,bps", [(1, 1, 1, 1), (333, 77, 1, 2), (1000, 70, 4, 1), (129, 40, 3, 2)])
def test_png_device_stays_in_its_length(engine, r2p, level, w, h, ch, bps):
    raw = np.random.default_rng(w * h + level).integers(0, 256, w * h * ch * bps, dtype=np.uint8)
    img = r2p.Image.make(w, h, ch, bps, r2p.WINDOW_NONE, level=level)
    cap = r2p.png_bound(img)
    out = Guarded(r2p, cap)
    ln = Guarded(r2p, 8)
    src = r2p.DeviceBuffer.from_array(raw)          # held until the results are read back
    engine.encode_png_device(img, src.ptr, out.ptr, cap, ln.ptr)
    n = int(np.frombuffer(ln.check(8), np.uint64)[0])
    assert 0 < n <= cap
    png = out.check(n)
    assert png == engine.encode_png(img, raw)


@pytest.mark.parametrize("w,h,ch,bps", [(1, 1, 1, 1), (7, 5, 3, 2), (4097, 3, 1, 1), (301, 33, 4, 2)])
def test_filter_device_stays_in_its_size(engine, r2p, w, h, ch, bps):
    raw = np.random.default_rng(w + h).integers(0, 256, w * h * ch * bps, dtype=np.uint8)
    img = r2p.Image.make(w, h, ch, bps, r2p.WINDOW_NONE)
    out = Guarded(r2p, img.filtered_bytes)
    last = Guarded(r2p, w * ch * bps)
    src = r2p.DeviceBuffer.from_array(raw)
    engine.window_filter_device(img, src.ptr, out.ptr, d_last_row=last.ptr)
    out.check(img.filtered_bytes)
    assert last.check(w * ch * bps) == raw.reshape(h, -1)[-1].tobytes()


@pytest.mark.parametrize("level", [0, 1, 6])
@pytest.mark.parametrize("n", [1, 4097, 65520, 200001])
def test_deflate_outputs_stay_in_their_length(engine, r2p, level, n):
    data = np.repeat(np.random.default_rng(n).integers(0, 9, n // 3 + 1, dtype=np.uint8), 3)[:n]
    src = r2p.DeviceBuffer.from_array(data)
    cap = r2p.zlib_bound(n, level)
    out, ln = Guarded(r2p, cap), Guarded(r2p, 8)
    engine.zlib_compress_device(src.ptr, n, level, out.ptr, cap, ln.ptr)
    m = int(np.frombuffer(ln.check(8), np.uint64)[0])
    import zlib
    assert zlib.decompress(out.check(m)) == data.tobytes()
    # raw part: the stream, then 4 bytes of Adler-32
    out2, ln2 = Guarded(r2p, cap), Guarded(r2p, 8)
    r2p.check(r2p.lib().r2p_deflate_raw_device(engine.h, src.ptr, n, level, 0, 0, out2.ptr, cap, ln2.ptr, None))
    m2 = int(np.frombuffer(ln2.check(8), np.uint64)[0])
    out2.check(m2 + 4)


def test_bmp_device_writes_exactly_the_file(engine, r2p):
    for (w, h, ch, bps) in ((1, 1, 1, 1), (7, 3, 3, 2), (13, 5, 1, 2), (6, 4, 4, 2)):
        raw = np.random.default_rng(w * h).integers(0, 256, w * h * ch * bps, dtype=np.uint8)
        img = r2p.Image.make(w, h, ch, bps, r2p.WINDOW_NONE)
        size = r2p.bmp_bound(img)
        out = Guarded(r2p, size)
        src = r2p.DeviceBuffer.from_array(raw)
        engine.encode_bmp_device(img, src.ptr, out.ptr, size)
        assert out.check(size) == engine.encode_bmp(img, raw)
        src.close()


def test_batch_outputs_stay_in_their_lengths(engine, r2p, W):
    imgs, outs, lens, srcs = [], [], [], []
    for i, (w, h, lvl) in enumerate([(300, 200, 1), (64, 64, 0), (1000, 300, 6), (5, 3, 1)]):
        raw = W.ct_phantom(50 + i, w, h)
        img = W.image_ct8(w, h, 40.0, 400.0, level=lvl)
        imgs.append(img)
        srcs.append(r2p.DeviceBuffer.from_array(raw))
        outs.append(Guarded(r2p, r2p.png_bound(img)))
    ln = Guarded(r2p, 8 * len(imgs))
    engine.encode_batch_device(imgs, [s.ptr for s in srcs], [o.ptr for o in outs], [o.n for o in outs], ln.ptr)
    n = np.frombuffer(ln.check(8 * len(imgs)), np.uint64)
    for i, o in enumerate(outs):
        assert 0 < int(n[i]) <= o.n
        o.check(int(n[i]))


def test_bounded_wait_runs_out_and_context_stays_usable(engine, r2p):
    # a barrier nothing completes: the kernel gives up after the limit and says so
    assert r2p.selftest_bounded_wait(arrive=False, limit_us=20000) == r2p.ETIMEOUT
    # one arrival completes it
    assert r2p.selftest_bounded_wait(arrive=True, limit_us=20000) == r2p.OK
    with pytest.raises(r2p.R2PError):
        r2p.selftest_bounded_wait(arrive=False, limit_us=0)
    # the context still encodes
    raw = np.arange(64 * 32, dtype=np.uint8)
    img = r2p.Image.make(64, 32, 1, 1, r2p.WINDOW_NONE, level=1)
    assert engine.encode_png(img, raw)[:8] == b"\x89PNG\r\n\x1a\n"


def test_engine_held_to_its_budget(r2p, W):
    with r2p.Engine(0, hbm_budget=16 << 20) as eng:
        big = W.image_c1(level=1)                       # 3072x3072: far more than 16 MB of work space
        with pytest.raises(r2p.R2PError) as ei:
            eng.encode_png(big, np.zeros(3072 * 3072, "<u2"))
        assert ei.value.status == r2p.EBUDGET
        small = r2p.Image.make(256, 128, 1, 1, r2p.WINDOW_NONE, level=1)
        assert eng.encode_png(small, np.zeros(256 * 128, np.uint8))[:4] == b"\x89PNG"
