"""Seeded synthetic inputs for the five benchmark workloads.

The reference names no public dataset, so every workload is generated here:
value noise from a splitmix64 stream, seed = 1000 * config + image index.

Per channel c and octave o = 0..3 (theta, phi ~ U[0, 2 pi)):
    v = 128 + sum_o (48 / 2^o) sin(2 pi (4 * 2^o) (x cos th + y sin th) / W + phi) + U[-16, 16)
clamped to [0, 255] and truncated to uint8.

Workloads (image sizes as named):
  heal256      256x256 RGB heal, centred 64x64 hole, brushfire order, P=30, trys=200
  render1024   128x128 RGBA tile (noise + tileable stripes) -> 1024x1024 target, random order,
               P=16, trys=300, no context
  heal4096     4096x4096 RGB heal, mask = union of 40 ellipses (10% +- 1% area), P=30, trys=200
  batch512     512 heal requests, 128..1024 square-ish sizes, Gray/RGB/RGBA, masks 2..20 %
  mapstyle2048 512x512 RGB corpus + blurred-luma map -> 2048x2048 target guided by a
               smooth grey map, mapWeight=0.5, P=30, trys=200, no context
"""
from __future__ import annotations

import math

import numpy as np

T_RGB, T_RGBA, T_Gray, T_GrayA = 0, 1, 2, 3
PIXELELS = {T_RGB: 3, T_RGBA: 4, T_Gray: 1, T_GrayA: 2}

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


class SplitMix64:
    """splitmix64 stream (Steele, Lea, Flood 2014), vectorised with numpy."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self.count = np.uint64(0)

    def next_u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            k = np.arange(1, n + 1, dtype=np.uint64) + self.count
            z = self.state + k * _GOLDEN
            self.count += np.uint64(n)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            return z ^ (z >> np.uint64(31))

    def uniform(self, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        u = (self.next_u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def integers(self, n: int, lo: int, hi: int) -> np.ndarray:
        """Uniform integers in [lo, hi]."""
        return (lo + np.floor(self.uniform(n) * (hi - lo + 1))).astype(np.int64)


def value_noise(h: int, w: int, channels: int, rng: SplitMix64, stripes: bool = False) -> np.ndarray:
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    out = np.empty((h, w, channels), np.uint8)
    for c in range(channels):
        v = np.full((h, w), 128.0)
        for o in range(4):
            th, ph = rng.uniform(2, 0.0, 2 * math.pi)
            f = 4 * 2 ** o
            v += (48.0 / 2 ** o) * np.sin(2 * math.pi * f * (x * math.cos(th) + y * math.sin(th)) / w + ph)
        if stripes:
            kx, ky = 0, 0
            while kx == 0 and ky == 0:
                kx, ky = (int(k) for k in rng.integers(2, -4, 4))
            v += 40.0 * np.sin(2 * math.pi * (kx * x + ky * y) / w)
        v += rng.uniform(h * w, -16.0, 16.0).reshape(h, w)
        out[..., c] = np.clip(v, 0, 255).astype(np.uint8)
    return out


def value_noise_fast(h: int, w: int, channels: int, rng: SplitMix64) -> np.ndarray:
    """value_noise (no stripes) in float64 through sin(a + b) = sin a cos b +
    cos a sin b: two 1-D evaluations and an outer product per octave, the same
    draws in the same order; for large images."""
    x = np.arange(w, dtype=np.float64)
    y = np.arange(h, dtype=np.float64)
    out = np.empty((h, w, channels), np.uint8)
    for c in range(channels):
        v = np.full((h, w), 128.0)
        for o in range(4):
            th, ph = rng.uniform(2, 0.0, 2 * math.pi)
            f = 2 * math.pi * (4 * 2 ** o) / w
            ax = f * math.cos(th) * x
            by = f * math.sin(th) * y + ph
            v += (48.0 / 2 ** o) * (np.outer(np.cos(by), np.sin(ax)) + np.outer(np.sin(by), np.cos(ax)))
        v += rng.uniform(h * w, -16.0, 16.0).reshape(h, w)
        out[..., c] = np.clip(v, 0, 255).astype(np.uint8)
    return out


def value_noise_separable(h: int, w: int, channels: int, rng: SplitMix64) -> np.ndarray:
    """value_noise's distribution, computed with sin(a + b) = sin a cos b + cos a sin b
    so each octave costs two 1-D trig evaluations and one outer product."""
    x = np.arange(w, dtype=np.float32)
    y = np.arange(h, dtype=np.float32)
    out = np.empty((h, w, channels), np.uint8)
    for c in range(channels):
        v = np.full((h, w), 128.0, np.float32)
        for o in range(4):
            th, ph = rng.uniform(2, 0.0, 2 * math.pi)
            f = 2 * math.pi * (4 * 2 ** o) / w
            ax = f * math.cos(th) * x
            by = f * math.sin(th) * y + ph
            amp = np.float32(48.0 / 2 ** o)
            v += amp * (np.outer(np.cos(by), np.sin(ax)) + np.outer(np.sin(by), np.cos(ax)))
        v += rng.uniform(h * w, -16.0, 16.0).reshape(h, w).astype(np.float32)
        out[..., c] = np.clip(v, 0, 255).astype(np.uint8)
    return out


def ellipse_mask_fast(h: int, w: int, rng: SplitMix64, count: int, rmin: float, rmax: float,
                      lo_frac: float, hi_frac: float, rects: bool = False) -> np.ndarray:
    """ellipse_mask with each shape rasterised only inside its bounding box;
    after 200 draws the one closest to the requested area is kept."""
    best, best_gap = None, None
    for _ in range(200):
        m = np.zeros((h, w), bool)
        for _ in range(count):
            cx, cy = rng.uniform(1, 0, w)[0], rng.uniform(1, 0, h)[0]
            rx, ry = rng.uniform(2, rmin, rmax)
            r = max(rx, ry)
            x0, x1 = max(0, int(cx - r) - 1), min(w, int(cx + r) + 2)
            y0, y1 = max(0, int(cy - r) - 1), min(h, int(cy + r) + 2)
            if x0 >= x1 or y0 >= y1:
                continue
            yy, xx = np.mgrid[y0:y1, x0:x1].astype(np.float32)
            if rects and rng.uniform(1)[0] < 0.5:
                m[y0:y1, x0:x1] |= (np.abs(xx - cx) < rx) & (np.abs(yy - cy) < ry)
            else:
                a = rng.uniform(1, 0, math.pi)[0]
                ca, sa = math.cos(a), math.sin(a)
                u = (xx - cx) * ca + (yy - cy) * sa
                v = -(xx - cx) * sa + (yy - cy) * ca
                m[y0:y1, x0:x1] |= (u / rx) ** 2 + (v / ry) ** 2 <= 1.0
        frac = m.mean()
        if lo_frac <= frac <= hi_frac:
            return np.where(m, 255, 0).astype(np.uint8)
        gap = min(abs(frac - lo_frac), abs(frac - hi_frac))
        if frac > 0 and (best_gap is None or gap < best_gap):
            best, best_gap = m, gap
    if best is None:
        raise RuntimeError("could not draw a mask")
    return np.where(best, 255, 0).astype(np.uint8)


def ellipse_mask(h: int, w: int, rng: SplitMix64, count: int, rmin: float, rmax: float,
                 lo_frac: float, hi_frac: float, rects: bool = False) -> np.ndarray:
    """Union of random ellipses (or rectangles), redrawn until the area lies in
    [lo_frac, hi_frac].  Each shape is evaluated only inside its bounding box
    (it covers no pixel outside it)."""
    for _ in range(200):
        m = np.zeros((h, w), bool)
        for _ in range(count):
            cx, cy = rng.uniform(1, 0, w)[0], rng.uniform(1, 0, h)[0]
            rx, ry = rng.uniform(2, rmin, rmax)
            r = max(rx, ry)
            x0, x1 = max(0, int(cx - r) - 1), min(w, int(cx + r) + 2)
            y0, y1 = max(0, int(cy - r) - 1), min(h, int(cy + r) + 2)
            y, x = np.mgrid[y0:y1, x0:x1].astype(np.float32)
            if rects and rng.uniform(1)[0] < 0.5:
                m[y0:y1, x0:x1] |= (np.abs(x - cx) < rx) & (np.abs(y - cy) < ry)
            else:
                a = rng.uniform(1, 0, math.pi)[0]
                ca, sa = math.cos(a), math.sin(a)
                u = (x - cx) * ca + (y - cy) * sa
                v = -(x - cx) * sa + (y - cy) * ca
                m[y0:y1, x0:x1] |= (u / rx) ** 2 + (v / ry) ** 2 <= 1.0
        frac = m.mean()
        if lo_frac <= frac <= hi_frac:
            return np.where(m, 255, 0).astype(np.uint8)
    raise RuntimeError("could not draw a mask with the requested area")


def heal256(index: int = 0) -> dict:
    """Plain heal of a 256x256 RGB image, centred 64x64 hole (4096 target px)."""
    rng = SplitMix64(1000 * 0 + index)
    img = value_noise(256, 256, 3, rng)
    mask = np.zeros((256, 256), np.uint8)
    mask[96:160, 96:160] = 255
    return dict(name="heal256", image=img, mask=mask, fmt=T_RGB,
                params=dict(matchContextType=2, patchSize=30, maxProbeCount=200, sensitivity=0.117),
                target_px=4096)


def heal_small(size: int = 48, hole: int = 12, fmt: int = T_RGB, ctype: int = 2, patch: int = 30,
               trys: int = 200, index: int = 0) -> dict:
    """Scaled-down heal256 for quick parity checks."""
    rng = SplitMix64(100000 + 1000 * fmt + index)
    img = value_noise(size, size, PIXELELS[fmt], rng)
    if fmt in (T_RGBA, T_GrayA):
        img[..., -1] = 255
    mask = np.zeros((size, size), np.uint8)
    a = (size - hole) // 2
    mask[a:a + hole, a:a + hole] = 255
    return dict(name=f"heal{size}", image=img, mask=mask, fmt=fmt,
                params=dict(matchContextType=ctype, patchSize=patch, maxProbeCount=trys, sensitivity=0.117),
                target_px=hole * hole)


def pixmap(colors: np.ndarray, mask: np.ndarray, alpha: np.ndarray | None = None,
           mapch: np.ndarray | None = None) -> np.ndarray:
    """Interleaves [mask][colors][alpha?][map...] (lib/imageFormat.c:116-207)."""
    h, w = mask.shape
    parts = [mask.reshape(h, w, 1), colors.reshape(h, w, -1)]
    if alpha is not None:
        parts.append(alpha.reshape(h, w, 1))
    if mapch is not None:
        parts.append(mapch.reshape(h, w, -1))
    return np.ascontiguousarray(np.concatenate(parts, axis=2).astype(np.uint8))


def render(tile: int = 128, out: int = 1024, index: int = 0) -> dict:
    """Render-texture enlarge: RGBA tile -> out x out RGBA target, no context.
    Format = prepareImageFormatIndices(3 colours, 0 map, alpha target, alpha corpus, no map)."""
    rng = SplitMix64(1000 * 1 + index)
    col = value_noise(tile, tile, 3, rng, stripes=True)
    alpha = np.full((tile, tile), 255, np.uint8)
    corpus = pixmap(col, np.full((tile, tile), 255, np.uint8), alpha)
    target = pixmap(np.zeros((out, out, 3), np.uint8), np.full((out, out), 255, np.uint8),
                    np.full((out, out), 255, np.uint8))
    return dict(name=f"render{out}", corpus=corpus, target=target, format=(3, 0, 1, 1, 0),
                params=dict(matchContextType=0, patchSize=16, maxProbeCount=300, sensitivity=0.117),
                target_px=out * out)


def render1024(index: int = 0) -> dict:
    return render(128, 1024, index)


def heal4096(index: int = 0, size: int = 4096) -> dict:
    rng = SplitMix64(1000 * 2 + index)
    img = value_noise_fast(size, size, 3, rng)
    scale = size / 4096.0
    mask = ellipse_mask(size, size, rng, 40, 20 * scale, 200 * scale, 0.09, 0.11)
    return dict(name=f"heal{size}", image=img, mask=mask, fmt=T_RGB,
                params=dict(matchContextType=1, patchSize=30, maxProbeCount=200, sensitivity=0.117),
                target_px=int((mask > 0).sum()))


def batch_specs(n: int = 512, lo: int = 128, hi: int = 1024, index: int = 0) -> list[dict]:
    """The per-request draws of batch_requests (size, layout, hole fraction,
    patch size), in request order; batch_request() makes one request's images
    from its spec, so requests can be generated in parallel."""
    rng = SplitMix64(1000 * 3 + index)
    specs = []
    for r in range(n):
        w, h = (int(v) for v in rng.integers(2, lo, hi))
        fmt = [T_Gray, T_RGB, T_RGBA][int(rng.integers(1, 0, 2)[0])]
        frac = float(rng.uniform(1, 0.02, 0.20)[0])
        patch = [9, 16, 30][int(rng.integers(1, 0, 2)[0])]
        specs.append(dict(r=r, w=w, h=h, fmt=fmt, frac=frac, patch=patch, index=index))
    return specs


def batch_request(spec: dict) -> dict:
    r, w, h, fmt, frac, index = spec["r"], spec["w"], spec["h"], spec["fmt"], spec["frac"], spec["index"]
    sub = SplitMix64(1000 * 3 + 7919 * (r + 1) + index)
    img = value_noise_separable(h, w, PIXELELS[fmt], sub)
    if fmt == T_RGBA:
        img[..., 3] = 255
    rmax = max(8.0, 0.25 * min(w, h))
    mask = ellipse_mask_fast(h, w, sub, 1 + int(frac * 40), 4.0, rmax, frac * 0.8, frac * 1.25, rects=True)
    return dict(name=f"req{r}", image=img, mask=mask, fmt=fmt,
                params=dict(matchContextType=1, patchSize=spec["patch"], maxProbeCount=200, sensitivity=0.117),
                target_px=int((mask > 0).sum()))


def batch_requests(n: int = 512, lo: int = 128, hi: int = 1024, index: int = 0) -> list[dict]:
    """Batched heal requests: sizes uniform in lo..hi per side, Gray/RGB/RGBA,
    holes of random ellipses and rectangles covering 2-20 %, P in {9, 16, 30}."""
    return [batch_request(sp) for sp in batch_specs(n, lo, hi, index)]


def gaussian_blur(a: np.ndarray, sigma: float) -> np.ndarray:
    r = int(math.ceil(3 * sigma))
    k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma) ** 2)
    k /= k.sum()
    p = np.pad(a.astype(np.float64), r, mode="reflect")
    p = np.apply_along_axis(lambda v: np.convolve(v, k, mode="valid"), 0, p)
    p = np.apply_along_axis(lambda v: np.convolve(v, k, mode="valid"), 1, p)
    return p


def mapstyle(corpus_size: int = 512, out: int = 2048, index: int = 0) -> dict:
    """Map-guided style transfer: internal pixel M,R,G,B,W
    (prepareImageFormatIndices(3 colours, 1 map colour, no alpha, no alpha, map))."""
    rng = SplitMix64(1000 * 4 + index)
    col = value_noise(corpus_size, corpus_size, 3, rng)
    luma = (77 * col[..., 0].astype(np.int32) + 150 * col[..., 1] + 29 * col[..., 2]) >> 8
    cmap = np.clip(gaussian_blur(luma, 4.0), 0, 255).astype(np.uint8)
    y, x = np.mgrid[0:out, 0:out].astype(np.float64) / out
    g = np.zeros((out, out))
    for _ in range(3):
        a = rng.uniform(1, 0, 2 * math.pi)[0]
        g += x * math.cos(a) + y * math.sin(a)
    f, ph, a = rng.uniform(3, 0, 1)
    g += 0.5 * np.sin(2 * math.pi * (1 + 2 * f) * (x * math.cos(6.28 * a) + y * math.sin(6.28 * a)) + 6.28 * ph)
    g = (g - g.min()) / max(1e-9, g.max() - g.min())
    tmap = (g * 255).astype(np.uint8)
    corpus = pixmap(col, np.full((corpus_size, corpus_size), 255, np.uint8), None, cmap)
    target = pixmap(np.zeros((out, out, 3), np.uint8), np.full((out, out), 255, np.uint8), None, tmap)
    return dict(name=f"mapstyle{out}", corpus=corpus, target=target, format=(3, 1, 0, 0, 1),
                params=dict(matchContextType=0, patchSize=30, maxProbeCount=200, sensitivity=0.117,
                            mapWeight=0.5),
                target_px=out * out)


def simple_to_pixmaps(image: np.ndarray, mask: np.ndarray, mask2: np.ndarray | None = None):
    """The simple-API adaption (lib/adaptSimple.h:260-354): target = image with
    its mask, corpus = image with the inverted mask (or mask2)."""
    h, w = mask.shape
    img = image.reshape(h, w, -1)
    target = np.concatenate([mask.reshape(h, w, 1), img], axis=2).astype(np.uint8)
    cm = (~mask).astype(np.uint8) if mask2 is None else mask2
    corpus = np.concatenate([cm.reshape(h, w, 1), img], axis=2).astype(np.uint8)
    return np.ascontiguousarray(target), np.ascontiguousarray(corpus)
