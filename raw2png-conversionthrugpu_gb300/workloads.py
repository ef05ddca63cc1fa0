"""Seeded synthetic inputs shaped like the five benchmark workloads.

The reference's own dataset (a CT folder) is not available; these generators
stand in for it with the stated shapes, bit depths and value distributions:
  ct_phantom      512x512 (or any size) 12-bit CT slice: background 0, body
                  ellipse 1064, six inner ellipses U[900, 2200], N(0, 20)
                  noise, clipped to [0, 4095]
  radial_rects    3072x3072 12-bit radial gradient 0..4095 + N(0, 8) noise +
                  40 constant rectangles
  rgb_sinusoids   6000x4000 RGB16: per channel 8 low-frequency 2-D sinusoids
                  scaled to [0, 65535] + N(0, 150), big-endian samples
  mixed_batch     1000 CT slices, sides from {256^2, 512^2, 1024^2,
                  2048x2500, 3072^2}, WC ~ U[-600, 400], WW ~ U[80, 1600]
  request_stream  served requests: side log-uniform in [256, 4096], aspect in
                  [0.75, 1.33], half 8-bit windowed, half 16-bit
All generators return little-endian uint16 arrays (DICOM order) unless noted.
"""
import numpy as np

from . import DicomParams, Image, WINDOW_BATCH8, WINDOW_DICOM16, WINDOW_NONE


def _ellipse_mask(h, w, cy, cx, ry, rx):
    y = (np.arange(h, dtype=np.float32)[:, None] - cy) / ry
    x = (np.arange(w, dtype=np.float32)[None, :] - cx) / rx
    return (y * y + x * x) <= 1.0


def ct_phantom(seed=0, width=512, height=512, noise=20.0):
    rng = np.random.default_rng(seed)
    img = np.zeros((height, width), np.float32)
    cy, cx = height / 2.0, width / 2.0
    ry, rx = 0.40 * height, 0.44 * width
    img[_ellipse_mask(height, width, cy, cx, ry, rx)] = 1064.0
    for _ in range(6):
        ey = cy + rng.uniform(-0.5, 0.5) * ry
        ex = cx + rng.uniform(-0.5, 0.5) * rx
        ay = rng.uniform(0.05, 0.25) * ry
        ax = rng.uniform(0.05, 0.25) * rx
        img[_ellipse_mask(height, width, ey, ex, ay, ax)] = rng.uniform(900.0, 2200.0)
    img += rng.normal(0.0, noise, size=img.shape).astype(np.float32)
    return np.clip(np.rint(img), 0, 4095).astype("<u2")


def ct_params(wc=40.0, ww=400.0):
    """12-bit CT: slope 1, intercept -1024."""
    return DicomParams.make(16, 12, 11, 0, slope=1.0, intercept=-1024.0, wc=wc, ww=ww)


def radial_rects(seed=1, width=3072, height=3072, nrects=40):
    rng = np.random.default_rng(seed)
    y = np.arange(height, dtype=np.float32)[:, None] - height / 2.0
    x = np.arange(width, dtype=np.float32)[None, :] - width / 2.0
    r = np.sqrt(y * y + x * x)
    img = 4095.0 * r / r.max()
    img += rng.normal(0.0, 8.0, size=img.shape).astype(np.float32)
    for _ in range(nrects):
        h = int(rng.integers(height // 40, height // 6))
        w = int(rng.integers(width // 40, width // 6))
        y0 = int(rng.integers(0, height - h))
        x0 = int(rng.integers(0, width - w))
        img[y0:y0 + h, x0:x0 + w] = rng.uniform(0, 4095)
    return np.clip(np.rint(img), 0, 4095).astype("<u2")


def rgb_sinusoids(seed=2, width=6000, height=4000, noise=150.0):
    """RGB16 big-endian (PNG order), as the TIFF/RAW loaders deliver it."""
    rng = np.random.default_rng(seed)
    yy = np.arange(height, dtype=np.float32)[:, None]
    xx = np.arange(width, dtype=np.float32)[None, :]
    out = np.empty((height, width, 3), ">u2")
    for c in range(3):
        acc = np.zeros((height, width), np.float32)
        for _ in range(8):
            fy = rng.uniform(0.2, 3.0) * 2 * np.pi / height
            fx = rng.uniform(0.2, 3.0) * 2 * np.pi / width
            ph = rng.uniform(0, 2 * np.pi)
            amp = rng.uniform(0.3, 1.0)
            # sin(a + b) = sin a cos b + cos a sin b, separable in y and x
            a = fy * yy + ph
            b = fx * xx
            acc += amp * (np.sin(a) * np.cos(b) + np.cos(a) * np.sin(b))
        acc = (acc - acc.min()) / (acc.max() - acc.min()) * 65535.0
        acc += rng.normal(0.0, noise, size=acc.shape).astype(np.float32)
        out[:, :, c] = np.clip(np.rint(acc), 0, 65535).astype(np.uint16)
    return out


BATCH_SIZES = [(256, 256), (512, 512), (1024, 1024), (2048, 2500), (3072, 3072)]


def mixed_batch_specs(n=1000, seed=3):
    """(width, height, wc, ww, seed) per slice."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        w, h = BATCH_SIZES[int(rng.integers(0, len(BATCH_SIZES)))]
        specs.append((w, h, float(rng.uniform(-600, 400)), float(rng.uniform(80, 1600)), seed * 100003 + i))
    return specs


def request_specs(n, seed=4):
    """(width, height, eight_bit, wc, ww, seed) per served request."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        side = float(np.exp(rng.uniform(np.log(256), np.log(4096))))
        aspect = float(rng.uniform(0.75, 1.33))
        w = max(16, int(round(side * np.sqrt(aspect))))
        h = max(16, int(round(side / np.sqrt(aspect))))
        out.append((w, h, bool(rng.random() < 0.5), float(rng.uniform(-600, 400)), float(rng.uniform(80, 1600)),
                    seed * 100003 + i))
    return out


# image descriptors for each workload ------------------------------------
def image_c0():
    return Image.make(512, 512, 1, 2, WINDOW_BATCH8, ct_params(40.0, 400.0), level=0, strip_height=128)


def image_c1(level=1):
    p = DicomParams.make(16, 12, 11, 0, wc=2048.0, ww=4096.0)
    return Image.make(3072, 3072, 1, 2, WINDOW_DICOM16, p, level=level, strip_height=1024)


def image_c2(level=1):
    return Image.make(6000, 4000, 3, 2, WINDOW_NONE, None, level=level, strip_height=1024)


def image_ct8(width, height, wc, ww, level=1):
    return Image.make(width, height, 1, 2, WINDOW_BATCH8, ct_params(wc, ww), level=level, strip_height=1024)


def image_ct16(width, height, wc, ww, level=1):
    p = DicomParams.make(16, 12, 11, 0, slope=1.0, intercept=-1024.0, wc=wc, ww=ww)
    return Image.make(width, height, 1, 2, WINDOW_DICOM16, p, level=level, strip_height=1024)


def ct_phantom_torch(seed, width, height, device="cuda", noise=20.0):
    """ct_phantom's recipe drawn on the GPU with torch (same distributions,
    torch's generator): returns an int16 device tensor of LE 12-bit values."""
    import torch
    rng = np.random.default_rng(seed)
    cy, cx = height / 2.0, width / 2.0
    ry, rx = 0.40 * height, 0.44 * width
    y = torch.arange(height, device=device, dtype=torch.float32)[:, None]
    x = torch.arange(width, device=device, dtype=torch.float32)[None, :]

    def ell(ey, ex, ay, ax):
        return ((y - ey) / ay) ** 2 + ((x - ex) / ax) ** 2 <= 1.0

    img = torch.zeros((height, width), device=device, dtype=torch.float32)
    img[ell(cy, cx, ry, rx)] = 1064.0
    for _ in range(6):
        ey = cy + rng.uniform(-0.5, 0.5) * ry
        ex = cx + rng.uniform(-0.5, 0.5) * rx
        ay = rng.uniform(0.05, 0.25) * ry
        ax = rng.uniform(0.05, 0.25) * rx
        img[ell(ey, ex, ay, ax)] = float(rng.uniform(900.0, 2200.0))
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    img += torch.randn((height, width), device=device, generator=g) * noise
    return torch.clamp(torch.round(img), 0, 4095).to(torch.int16)
