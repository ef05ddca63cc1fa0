"""Dynamic Huffman block builder (csrc/r2p_huff.h) on the host, no GPU.

tests/cpp/huff_check.cpp links the same header the GPU kernel uses.  Its code
lengths must cost exactly as much as a heap-built Huffman code whenever that
code fits 15 bits (and stay a complete code within 15 bits otherwise), and its
dynamic-Huffman DEFLATE streams must inflate with stock zlib to their input.
"""
import heapq
import os
import subprocess
import zlib

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def huff(tmp_path_factory):
    exe = tmp_path_factory.mktemp("huff") / "huff_check"
    subprocess.run(["g++", "-std=c++17", "-O2", "-o", str(exe), os.path.join(ROOT, "tests", "cpp", "huff_check.cpp")],
                   check=True)
    return str(exe)


def heap_lengths(freq):
    """Code lengths of a Huffman code built with a heap (no length limit)."""
    items = [(f, i, (i,)) for i, f in enumerate(freq) if f > 0]
    if len(items) == 1:
        return {items[0][1]: 1}
    depth = {i: 0 for _, i, _ in items}
    heapq.heapify(items)
    k = len(freq)
    while len(items) > 1:
        fa, _, a = heapq.heappop(items)
        fb, _, b = heapq.heappop(items)
        for s in a + b:
            depth[s] += 1
        heapq.heappush(items, (fa + fb, k, a + b))
        k += 1
    return depth


def test_lengths_optimal_and_limited(huff):
    rng = np.random.default_rng(1)
    cases = []
    for n in (2, 3, 5, 19, 30, 64, 286):
        for dist in ("uniform", "geometric", "sparse"):
            if dist == "uniform":
                f = rng.integers(1, 1000, n)
            elif dist == "geometric":
                f = np.maximum(1, (20000 * 0.7 ** np.arange(n)).astype(np.int64))
                rng.shuffle(f)
            else:
                f = rng.integers(0, 50, n) * (rng.random(n) < 0.3)
                f[rng.integers(0, n)] += 1
                f[(rng.integers(0, n) + 1) % n] += 1
            cases.append(f)
    cases.append(np.array([1, 1, 2, 3, 5, 8, 13, 21, 34, 55, 89, 144, 233, 377, 610, 987, 1597, 2584, 4181, 6765,
                           10946, 17711, 28657, 46368]))            # Fibonacci: optimal depth 23 > 15
    inp = "\n".join(" ".join(str(int(v)) for v in f) for f in cases) + "\n"
    out = subprocess.run([huff, "lengths"], input=inp, capture_output=True, text=True, check=True).stdout.split("\n")
    limited = 0
    for f, line in zip(cases, out):
        L = [int(x) for x in line.split()]
        used = [i for i, v in enumerate(f) if v > 0]
        assert all((L[i] > 0) == (f[i] > 0) for i in range(len(f)))
        assert max(L) <= 15
        if len(used) >= 2:
            assert sum(2.0 ** -L[i] for i in used) == 1.0, "complete prefix code"
        H = heap_lengths(list(f))
        best = sum(f[i] * H[i] for i in used)
        cost = sum(f[i] * L[i] for i in used)
        if max(H.values()) <= 15:
            assert cost == best
        else:
            limited += 1
            assert cost >= best
    assert limited >= 1


@pytest.mark.parametrize("kind", ["random", "runs", "filtered", "one", "tiny", "zeros"])
@pytest.mark.parametrize("blk", [65520, 1024])
def test_rle_dynamic_stream_inflates(huff, tmp_path, kind, blk):
    rng = np.random.default_rng(sum(kind.encode()))
    if kind == "random":
        data = rng.integers(0, 256, 150000, dtype=np.uint8)
    elif kind == "runs":
        data = np.repeat(rng.integers(0, 4, 3000, dtype=np.uint8), rng.integers(1, 300, 3000))
    elif kind == "filtered":     # small signed residuals, as PNG filtering leaves
        data = (np.round(rng.normal(0, 3, 200000)).astype(np.int64) % 256).astype(np.uint8)
        data[50000:90000] = 0
    elif kind == "one":
        data = np.array([7], np.uint8)
    elif kind == "tiny":
        data = np.array([1, 1, 1, 1, 2], np.uint8)
    else:
        data = np.zeros(100000, np.uint8)
    src, dst = tmp_path / "in.bin", tmp_path / "out.bin"
    data.tofile(src)
    subprocess.run([huff, "rle", str(src), str(dst), str(blk)], check=True)
    raw = dst.read_bytes()
    assert zlib.decompress(raw, -15) == data.tobytes()
    if kind == "filtered" and blk == 65520:
        c = zlib.compressobj(9, zlib.DEFLATED, -15, 9, zlib.Z_RLE)
        z = len(c.compress(data.tobytes()) + c.flush())
        assert len(raw) <= 1.02 * z, (len(raw), z)     # zlib's own RLE strategy as the yardstick
