"""Plug-in presets as request types: the host-side preparation that the
reference's Python-Fu scripts (PluginScripts/*.py) do in GIMP before calling
the engine plug-in, restated on numpy arrays so that each becomes one
synthesis request to this library.

`plug_in_resynthesizer` mirrors the engine plug-in's adaption
(src/resynthesizer/resynthesizer.c:380-513, adaptParameters.c): the target is
an image whose selected pixels are synthesized (the rest is context), the
corpus is a second image whose selected pixels may be copied, optional input
and output maps add map channels, and the seven numeric parameters map to
TImageSynthParameters one to one (h_tile, v_tile -> tiling, use_border ->
matchContextType, map_weight, autism -> sensitivityToOutliers, neighbours ->
patchSize, trys -> maxProbeCount).  Alpha is not matched: a totally
transparent corpus pixel is not in the corpus, and the target's alpha is
left as it is.

Images are uint8 arrays [H, W, C] (C = 1 grey, 2 grey+alpha, 3 RGB, 4 RGBA);
selections are [H, W] booleans (None = everything); maps are [H, W, C]
uint8 (their alpha, if any, is dropped).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import workloads as W


@dataclass
class PluginParameters:
    """The engine plug-in's numeric parameters (resynth-parameters.h)."""
    h_tile: int = 0
    v_tile: int = 0
    use_border: int = 1
    map_weight: float = 0.5
    autism: float = 0.117
    neighbours: int = 30
    trys: int = 200


def _split(image: np.ndarray):
    """(colours, alpha or None) of an [H, W, C] image."""
    img = image if image.ndim == 3 else image[..., None]
    c = img.shape[2]
    if c in (2, 4):
        return img[..., :c - 1], img[..., c - 1]
    return img, None


def _map_channels(m: np.ndarray | None):
    if m is None:
        return None
    colours, _ = _split(m)
    return colours


@dataclass
class Request:
    """One engine() call: interleaved target and corpus pixmaps, the
    prepareImageFormatIndices arguments and the parameters."""
    target: np.ndarray
    corpus: np.ndarray
    format: tuple
    params: dict


def plugin_request(image, selection, corpus, corpus_selection, p: PluginParameters, map_in=None,
                   map_out=None) -> Request:
    """The engine plug-in's adaption: pixmaps [mask][colours][alpha?][map...]
    with mask 255 on selected pixels, format from the channel counts."""
    tcol, talpha = _split(image)
    ccol, calpha = _split(corpus)
    if tcol.shape[2] != ccol.shape[2]:
        raise ValueError("the input texture and output image must have the same number of colour channels")
    h, w = tcol.shape[:2]
    ch, cw = ccol.shape[:2]
    with_map = map_in is not None and map_out is not None
    min_ = _map_channels(map_in) if with_map else None
    mout = _map_channels(map_out) if with_map else None
    if with_map:
        if min_.shape[2] != mout.shape[2]:
            raise ValueError("the input and output maps must have the same mode")
        if min_.shape[:2] != (ch, cw):
            raise ValueError("the input map should be the same size as the input texture image")
        if mout.shape[:2] != (h, w):
            raise ValueError("the output map should be the same size as the output image")
    tsel = np.ones((h, w), bool) if selection is None else np.asarray(selection, bool)
    csel = np.ones((ch, cw), bool) if corpus_selection is None else np.asarray(corpus_selection, bool)
    target = W.pixmap(tcol, np.where(tsel, 255, 0).astype(np.uint8), talpha, mout)
    corp = W.pixmap(ccol, np.where(csel, 255, 0).astype(np.uint8), calpha, min_)
    fmt = (tcol.shape[2], min_.shape[2] if with_map else 0, int(talpha is not None), int(calpha is not None),
           int(with_map))
    params = dict(tileH=p.h_tile, tileV=p.v_tile, matchContextType=p.use_border, mapWeight=float(p.map_weight),
                  sensitivity=float(p.autism), patchSize=min(int(p.neighbours), 64), maxProbeCount=int(p.trys))
    return Request(target, corp, fmt, params)


def apply_result(image, synthesized_target: np.ndarray) -> np.ndarray:
    """The image with its colour channels taken from the synthesized target pixmap."""
    img = image if image.ndim == 3 else image[..., None]
    nc = _split(img)[0].shape[2]
    out = img.copy()
    out[..., :nc] = synthesized_target[..., 1:1 + nc]
    return out if image.ndim == 3 else out[..., 0]


def run_request(req: Request, opts=None):
    """Runs a request through this library's engine(); returns the Result."""
    from . import engine, format_indices, params
    return engine(req.target, req.corpus, format_indices(*req.format), params(**req.params), opts=opts)


def plug_in_resynthesizer(image, selection, corpus, corpus_selection, p: PluginParameters, map_in=None,
                          map_out=None, opts=None):
    """Synthesizes the selected pixels of `image` from the selected pixels of
    `corpus` (None selections = everything); returns (rc, new image, Result)."""
    r = run_request(plugin_request(image, selection, corpus, corpus_selection, p, map_in, map_out), opts)
    return r.rc, apply_result(image, r.out), r


# ------------------------------------------------------------ selection ops

def grow(selection: np.ndarray, radius: int) -> np.ndarray:
    """Selection grown by `radius` pixels (a disc)."""
    sel = np.asarray(selection, bool)
    if radius <= 0:
        return sel.copy()
    from scipy import ndimage
    dist = ndimage.distance_transform_edt(~sel)
    return dist <= radius


def shrink(selection: np.ndarray, radius: int) -> np.ndarray:
    """Selection shrunk by `radius` pixels; the image border counts as unselected."""
    sel = np.asarray(selection, bool)
    if radius <= 0:
        return sel.copy()
    from scipy import ndimage
    dist = ndimage.distance_transform_edt(np.pad(sel, 1))[1:-1, 1:-1]
    return dist > radius


def bounds(selection: np.ndarray):
    """(x1, y1, x2, y2) of the selection, x2 and y2 exclusive, or None if empty."""
    ys, xs = np.nonzero(selection)
    if len(xs) == 0:
        return None
    return int(xs.min()), int(ys.min()), int(xs.max()) + 1, int(ys.max()) + 1


def resize(image: np.ndarray, width: int, height: int) -> np.ndarray:
    """Bilinear resample to width x height (pixel centres aligned)."""
    img = image.astype(np.float64) if image.ndim == 3 else image[..., None].astype(np.float64)
    h, w = img.shape[:2]
    ys = np.clip((np.arange(height) + 0.5) * h / height - 0.5, 0, h - 1)
    xs = np.clip((np.arange(width) + 0.5) * w / width - 0.5, 0, w - 1)
    y0 = np.floor(ys).astype(int)
    x0 = np.floor(xs).astype(int)
    y1, x1 = np.minimum(y0 + 1, h - 1), np.minimum(x0 + 1, w - 1)
    fy, fx = (ys - y0)[:, None, None], (xs - x0)[None, :, None]
    out = (img[y0][:, x0] * (1 - fy) * (1 - fx) + img[y0][:, x1] * (1 - fy) * fx +
           img[y1][:, x0] * fy * (1 - fx) + img[y1][:, x1] * fy * fx)
    out = np.clip(np.rint(out), 0, 255).astype(np.uint8)
    return out if image.ndim == 3 else out[..., 0]


def grayscale(image: np.ndarray) -> np.ndarray:
    """Luminance of an RGB(A) image as [H, W, 1] (grey images unchanged)."""
    colours, _ = _split(image)
    if colours.shape[2] == 1:
        return colours.copy()
    c = colours.astype(np.uint32)
    return ((77 * c[..., 0] + 150 * c[..., 1] + 29 * c[..., 2]) >> 8).astype(np.uint8)[..., None]


# ------------------------------------------------------------------ presets

def heal_selection_request(image, selection, sampling_radius=50, direction=0, order=0):
    """PluginScripts/plugin-heal-selection.py:36-148.  The corpus is a donut
    of `sampling_radius` pixels around the selection (cut to the sides or to
    above and below by `direction`), the filling order random (0), inwards
    (1) or outwards (2).  Returns (corpus, corpus selection, parameters)."""
    sel = np.asarray(selection, bool)
    tb = bounds(sel)
    if tb is None:
        raise ValueError("you must first select a region to heal")
    grown = grow(sel, sampling_radius)
    donut = grown & ~sel
    fx1, fy1, fx2, fy2 = bounds(grown)
    tx1, ty1, tx2, ty2 = tb
    if direction == 0:     # all around
        nw, nh, nx, ny = fx2 - fx1, fy2 - fy1, fx1, fy1
    elif direction == 1:   # sides: target height, frisket width
        nw, nh, nx, ny = fx2 - fx1, ty2 - ty1, fx1, ty1
    else:                  # above and below: target width, frisket height
        nw, nh, nx, ny = tx2 - tx1, fy2 - fy1, tx1, fy1
    h, w = sel.shape
    nw, nh = min(w - nx, nw), min(h - ny, nh)
    corpus = image[ny:ny + nh, nx:nx + nw].copy()
    corpus_sel = donut[ny:ny + nh, nx:nx + nw].copy()
    use_border = 1 if not order else (direction + 2 if order == 1 else direction + 5)
    return corpus, corpus_sel, PluginParameters(0, 0, use_border, 0.0, 0.117, 16, 500)


def heal_selection(image, selection, sampling_radius=50, direction=0, order=0, opts=None):
    corpus, csel, p = heal_selection_request(image, selection, sampling_radius, direction, order)
    return plug_in_resynthesizer(image, selection, corpus, csel, p, opts=opts)


def heal_transparency(image, sampling_radius=50, order=2, background=255, opts=None):
    """PluginScripts/plugin-heal-transparency.py: heal the transparent pixels
    (selection = not opaque, grown by one pixel) of an image with alpha,
    after flattening it onto the background colour."""
    colours, alpha = _split(image)
    if alpha is None:
        return 0, image.copy(), None
    sel = grow(alpha < 255, 1)
    a = alpha.astype(np.uint32)[..., None]
    flat = ((colours.astype(np.uint32) * a + background * (255 - a) + 127) // 255).astype(np.uint8)
    return heal_selection(flat, sel, sampling_radius, 0, order, opts=opts)


def render_texture(image, selection=None, resize_ratio=2.0, make_tile=False, opts=None):
    """PluginScripts/plugin-render-texture.py: a new (white) image
    `resize_ratio` times the selection's size filled with texture
    synthesized from the selection; tileable if `make_tile`."""
    if selection is not None and bounds(selection) is not None:
        x1, y1, x2, y2 = bounds(selection)
    else:
        x1, y1, x2, y2 = 0, 0, image.shape[1], image.shape[0]
    nw, nh = int((x2 - x1) * resize_ratio), int((y2 - y1) * resize_ratio)
    colours, alpha = _split(image)
    new = np.full((nh, nw, image.shape[2] if image.ndim == 3 else 1), 255, np.uint8)
    corpus = image[y1:y2, x1:x2].copy()
    t = 1 if make_tile else 0
    p = PluginParameters(t, t, 0, 0.0, 0.117, 9, 200)
    new = new if image.ndim == 3 else new[..., 0]
    return plug_in_resynthesizer(new, None, corpus, None, p, opts=opts)


def fill_pattern(image, selection, pattern, opts=None):
    """PluginScripts/plugin-resynth-fill-pattern.py: fill the selection with
    texture synthesized from a pattern image."""
    p = PluginParameters(0, 0, 0, 0.0, 0.05, 8, 300)
    return plug_in_resynthesizer(image, selection, pattern, None, p, opts=opts)


def uncrop_request(image, percent=10):
    """PluginScripts/plugin-uncrop.py: the canvas grows by `percent` (centred);
    the new outer ring is the target and a band of the original's edge as wide
    as the growth is the corpus.  Returns (canvas, target selection, corpus,
    corpus selection, parameters)."""
    h, w = image.shape[:2]
    f = percent / 100.0 + 1.0
    nw, nh = int(w * f), int(h * f)
    ox, oy = int((nw - w) / 2), int((nh - h) / 2)
    canvas = np.zeros((nh, nw) + image.shape[2:], np.uint8)
    canvas[oy:oy + h, ox:ox + w] = image
    target_sel = np.ones((nh, nw), bool)
    target_sel[oy:oy + h, ox:ox + w] = False
    max_delta = max(w * percent / 100.0, h * percent / 100.0) / 2
    corpus_sel = ~shrink(np.ones((h, w), bool), int(max_delta))
    return canvas, target_sel, image.copy(), corpus_sel, PluginParameters(0, 0, 5, 0.0, 0.117, 16, 500)


def uncrop(image, percent=10, opts=None):
    canvas, tsel, corpus, csel, p = uncrop_request(image, percent)
    return plug_in_resynthesizer(canvas, tsel, corpus, csel, p, opts=opts)


def enlarge(image, scale_factor=2.0, opts=None):
    """PluginScripts/plugin-resynth-enlarge.py: scale up, then restore detail
    from the original (corpus), matching the scaled-up image (output map)
    against a blurred original (input map: scaled down and back up)."""
    h, w = image.shape[:2]
    small = resize(image, max(1, int(w / scale_factor)), max(1, int(h / scale_factor)))
    map_in = resize(small, w, h)
    big = resize(image, int(w * scale_factor), int(h * scale_factor))
    p = PluginParameters(0, 0, 0, 1.0, 0.117, 8, 500)
    return plug_in_resynthesizer(big, None, image, None, p, map_in=map_in, map_out=big, opts=opts)


def sharpen(image, scale_factor=2.0, opts=None):
    """PluginScripts/plugin-resynth-sharpen.py: resynthesize the image from a
    smaller copy (corpus), matching the image (output map) against that copy
    blurred (input map: halved and scaled back up)."""
    h, w = image.shape[:2]
    cw_, ch_ = max(1, int(w / scale_factor)), max(1, int(h / scale_factor))
    corpus = resize(image, cw_, ch_)
    map_in = resize(resize(image, max(1, int(w / (2 * scale_factor))), max(1, int(h / (2 * scale_factor)))), cw_, ch_)
    p = PluginParameters(0, 0, 0, 1.0, 0.117, 8, 500)
    return plug_in_resynthesizer(image, None, corpus, None, p, map_in=map_in, map_out=image, opts=opts)


def map_weight_for_transfer(percent_transfer: float) -> float:
    """PluginScripts/plugin-map-style.py calculate_map_weight: a sinusoid that
    linearises the map weight for the user's percent of style transfer."""
    return math.acos((percent_transfer / 100) * 2 - 1) / (2 * 3.14)


def map_style(image, style, percent_transfer=10.0, map_by_brightness=False, selection=None, opts=None):
    """PluginScripts/plugin-map-style.py transfer_style: re-render `image`
    with the texture of `style`, guided by maps (the images themselves, or
    their brightness for `map_by_brightness`, with the style's contrast moved
    toward the image's)."""
    tcol, _ = _split(image)
    scol, salpha = _split(style)
    if tcol.shape[2] != scol.shape[2]:
        # the plug-in upgrades grey to RGB rather than the reverse
        if tcol.shape[2] == 1:
            image = np.repeat(tcol, 3, axis=2)
        else:
            scol = np.repeat(scol, 3, axis=2)
    source = scol if salpha is None else np.concatenate([scol, salpha[..., None]], axis=2)
    if map_by_brightness:
        tmap = grayscale(image)
        smap = grayscale(source).astype(np.float64)
        # synchronize_contrast: shift the style map's contrast by the brightness difference
        control = (tmap.mean() - smap.mean()) * 2.5 * (1 - percent_transfer / 100)
        control = max(-127.0, min(127.0, control))
        slope = math.tan((control / 127.0 + 1) * math.pi / 4)
        smap = np.clip((smap - 127.5) * slope + 127.5, 0, 255).astype(np.uint8)
    else:
        tmap, smap = _split(image)[0], scol
    p = PluginParameters(1, 1, 1, map_weight_for_transfer(percent_transfer), 0.117, 9, 200)
    return plug_in_resynthesizer(image, selection, source, None, p, map_in=smap, map_out=tmap, opts=opts)
