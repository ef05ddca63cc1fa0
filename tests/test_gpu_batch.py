"""Batched encoding: one planned work list over many images, launched
directly or replayed as a CUDA graph, and size-class tuning.

Every PNG is decoded by the oracle's reader and compared with the oracle's
pixels and filtered scanlines (see test_gpu_png.decode_and_check); graph
replays and direct launches must give byte-identical files.
"""
import numpy as np
import pytest

from test_gpu_png import decode_and_check

pytestmark = pytest.mark.gpu


def make_batch_inputs(r2p, W, specs, level=1):
    imgs, raws, bufs, outs, caps = [], [], [], [], []
    for i, (w, h, wc, ww) in enumerate(specs):
        raw = W.ct_phantom(100 + i, w, h)
        img = W.image_ct8(w, h, wc, ww, level=level)
        imgs.append(img)
        raws.append(raw)
        bufs.append(r2p.DeviceBuffer.from_array(raw))
        caps.append(r2p.png_bound(img))
        outs.append(r2p.DeviceBuffer(caps[-1]))
    lens = r2p.DeviceBuffer(8 * len(imgs))
    return imgs, raws, bufs, outs, caps, lens


def read_all(outs, lens, n):
    ln = lens.download(8 * n).view(np.uint64)
    return [outs[i].download(int(ln[i])).tobytes() for i in range(n)]


SPECS = [(256, 256, 40.0, 400.0), (512, 512, -300.0, 1500.0), (1024, 64, 100.0, 90.0), (33, 7, 0.0, 800.0),
         (700, 300, -600.0, 250.0), (256, 256, 350.0, 1200.0)]


def test_batch_direct_and_graph(engine, O, r2p, W):
    imgs, raws, bufs, outs, caps, lens = make_batch_inputs(r2p, W, SPECS)
    b = engine.batch(imgs, [x.ptr for x in bufs], [o.ptr for o in outs], caps, lens.ptr)
    assert b.device_bytes > 0
    b.launch()
    direct = read_all(outs, lens, len(imgs))
    for i in range(len(imgs)):
        decode_and_check(O, r2p, imgs[i], raws[i], direct[i])
    for _ in range(2):
        for o in outs:
            o.memset(0)
        b.launch_graph()
        assert read_all(outs, lens, len(imgs)) == direct
    b.close()
    # the same images one call each give the same files
    for i in range(len(imgs)):
        assert engine.encode_png(imgs[i], raws[i]) == direct[i]


def test_tuning_table_changes_blocks_not_pixels(O, r2p, W):
    eng = r2p.Engine(0)
    eng.set_tuning([(300000, 4096, 8, 9), (2 ** 40, 32752, 0, 10)])
    assert eng.get_tuning()[0] == (300000, 4096, 8, 9)
    imgs, raws, bufs, outs, caps, lens = make_batch_inputs(r2p, W, SPECS)
    b = eng.batch(imgs, [x.ptr for x in bufs], [o.ptr for o in outs], caps, lens.ptr)
    b.launch_graph()
    pngs = read_all(outs, lens, len(imgs))
    for i in range(len(imgs)):
        decode_and_check(O, r2p, imgs[i], raws[i], pngs[i])
    b.close()
    with pytest.raises(r2p.R2PError):
        eng.set_tuning([(100, 4096, 0, 11)])
    eng.set_tuning([])
    builtin = eng.get_tuning()
    assert builtin[-1][1] == 21760 and all(c[1] == 21760 for c in builtin)   # the GB300 autotuned table
    eng.close()


def test_tuned_block_size_applies_to_level_1_only(engine, r2p, W):
    """The table's block size is the LZ77 kernel's: a level-1 image follows it,
    stored (level 0) and dynamic-Huffman (level 6) images keep 65520-byte
    blocks, so their bytes match an engine with the built-in table."""
    eng = r2p.Engine(0)
    eng.set_tuning([(2 ** 62, 4096, 0, 10)])
    raw = W.ct_phantom(77, 640, 480)
    for level in (0, 1, 6):
        img = W.image_ct8(640, 480, 40.0, 400.0, level=level)
        same = eng.encode_png(img, raw) == engine.encode_png(img, raw)
        assert same == (level != 1), level
    eng.close()


@pytest.mark.parametrize("small,large", [(32752, 65520), (21760, 32752), (21760, 65520), (4096, 21760)])
def test_mixed_tuning_classes_same_as_alone(O, r2p, W, small, large):
    """Images of different size classes (different block sizes and LZ77 table
    sizes) in one batch give the same bytes as each image encoded alone: the
    launch picks its CTA size (1024, 512 or 320 threads) for the largest
    block, and a block's bytes must not depend on it."""
    eng = r2p.Engine(0)
    eng.set_tuning([(200000, small, 0, 9), (2 ** 40, large, 0, 10)])
    specs = [(256, 256, 40.0, 400.0), (700, 600, -300.0, 1500.0), (300, 200, 100.0, 90.0), (640, 640, 0.0, 800.0)]
    imgs, raws, bufs, outs, caps, lens = make_batch_inputs(r2p, W, specs)
    b = eng.batch(imgs, [x.ptr for x in bufs], [o.ptr for o in outs], caps, lens.ptr)
    b.launch_graph()
    pngs = read_all(outs, lens, len(imgs))
    b.close()
    for i in range(len(imgs)):
        assert pngs[i] == eng.encode_png(imgs[i], raws[i]), "image %d differs between batch and alone" % i
        decode_and_check(O, r2p, imgs[i], raws[i], pngs[i])
    eng.close()


def test_dynamic_level_batch_equals_alone(engine, O, r2p, W):
    # a few blocks alone run the dynamic kernel with 1024-thread CTAs; a batch
    # of many blocks runs it with 512-thread CTAs: the files must not differ
    specs = SPECS + [(3072, 2048, 40.0, 400.0), (2048, 2500, -100.0, 700.0)]
    imgs, raws, bufs, outs, caps, lens = make_batch_inputs(r2p, W, specs, level=6)
    engine.encode_batch_device(imgs, [x.ptr for x in bufs], [o.ptr for o in outs], caps, lens.ptr)
    batched = read_all(outs, lens, len(imgs))
    for i in range(len(imgs)):
        decode_and_check(O, r2p, imgs[i], raws[i], batched[i])
        assert engine.encode_png(imgs[i], raws[i]) == batched[i], specs[i]


def test_split_batch_graph_equals_alone(engine, O, r2p, W):
    # 80 images: the batch runs as four size-balanced parts, parallel branches
    # of one graph; every file must equal the image encoded alone
    rng = np.random.default_rng(5)
    specs = [(int(rng.integers(16, 400)), int(rng.integers(4, 300)), float(rng.uniform(-300, 300)),
              float(rng.uniform(80, 1500))) for _ in range(80)]
    imgs, raws, bufs, outs, caps, lens = make_batch_inputs(r2p, W, specs, level=1)
    for i in range(0, len(imgs), 3):
        imgs[i].level = 6 if i % 2 else 0
        caps[i] = r2p.png_bound(imgs[i])
        outs[i] = r2p.DeviceBuffer(caps[i])
    b = engine.batch(imgs, [x.ptr for x in bufs], [o.ptr for o in outs], caps, lens.ptr)
    b.launch_graph()
    graphed = read_all(outs, lens, len(imgs))
    for o in outs:
        o.memset(0)
    b.launch()
    assert read_all(outs, lens, len(imgs)) == graphed
    b.close()
    for i in range(len(imgs)):
        assert engine.encode_png(imgs[i], raws[i]) == graphed[i], specs[i]
        if i % 10 == 0:
            decode_and_check(O, r2p, imgs[i], raws[i], graphed[i])
