"""Plug-in presets (PluginScripts/*.py) as requests: their preparation
(selections, crops, maps, parameters) on the CPU, and the CPU engine run on
small requests.  The GPU runs of the same requests are in
tests/test_gpu_presets.py."""
import math

import numpy as np
import pytest

from oracle import make_params
from resynthesizer_gb300 import presets as PR
from resynthesizer_gb300 import workloads as W


def _image(h, w, c, seed):
    return W.value_noise(h, w, c, W.SplitMix64(seed))


def _disc(h, w, cx, cy, r):
    y, x = np.mgrid[0:h, 0:w]
    return (x - cx) ** 2 + (y - cy) ** 2 <= r * r


@pytest.mark.parametrize("direction,order,border", [(0, 0, 1), (1, 0, 1), (0, 1, 2), (1, 1, 3), (2, 1, 4),
                                                    (0, 2, 5), (1, 2, 6), (2, 2, 7)])
def test_heal_selection_request(direction, order, border):
    img = _image(60, 80, 3, 1)
    sel = _disc(60, 80, 40, 30, 6)
    corpus, csel, p = PR.heal_selection_request(img, sel, sampling_radius=10, direction=direction, order=order)
    assert (p.use_border, p.neighbours, p.trys, p.autism, p.map_weight) == (border, 16, 500, 0.117, 0.0)
    x1, y1, x2, y2 = PR.bounds(sel)
    g = PR.grow(sel, 10)
    fx1, fy1, fx2, fy2 = PR.bounds(g)
    if direction == 0:
        assert corpus.shape[:2] == (fy2 - fy1, fx2 - fx1)
    elif direction == 1:
        assert corpus.shape[:2] == (y2 - y1, fx2 - fx1)
    else:
        assert corpus.shape[:2] == (fy2 - fy1, x2 - x1)
    # the corpus never contains the target, and only pixels within the sampling radius
    ox = fx1 if direction != 2 else x1
    oy = fy1 if direction != 1 else y1
    full = np.zeros_like(sel)
    full[oy:oy + csel.shape[0], ox:ox + csel.shape[1]] = csel
    assert not (full & sel).any() and (full <= g).all() and full.any()
    assert np.array_equal(corpus, img[oy:oy + csel.shape[0], ox:ox + csel.shape[1]])


def test_grow_shrink_bounds():
    sel = np.zeros((20, 20), bool)
    sel[10, 10] = True
    g = PR.grow(sel, 3)
    assert g.sum() == 29 and PR.bounds(g) == (7, 7, 14, 14)     # disc of radius 3
    s = PR.shrink(np.ones((20, 30), bool), 4)
    assert PR.bounds(s) == (4, 4, 26, 16)


def test_uncrop_request():
    img = _image(40, 50, 3, 2)
    canvas, tsel, corpus, csel, p = PR.uncrop_request(img, percent=20)
    assert canvas.shape[:2] == (48, 60) and p.use_border == 5 and (p.neighbours, p.trys) == (16, 500)
    assert np.array_equal(canvas[4:44, 5:55], img) and tsel.sum() == 48 * 60 - 40 * 50
    # corpus: a band of the original's edge, max(50, 40) * 20 % / 2 = 5 px wide
    assert csel[0].all() and csel[:, 0].all() and not csel[5:35, 5:45].any() and csel[4, 20]


def test_render_texture_and_maps():
    assert math.isclose(PR.map_weight_for_transfer(50), math.acos(0) / (2 * 3.14))
    assert PR.map_weight_for_transfer(100) == 0.0
    img = _image(30, 40, 3, 3)
    req = PR.plugin_request(np.full((60, 80, 3), 255, np.uint8), None, img, None, PR.PluginParameters(1, 1, 0, 0.0, 0.117, 9, 200))
    assert req.format == (3, 0, 0, 0, 0) and req.target.shape == (60, 80, 4) and (req.target[..., 0] == 255).all()
    assert req.params == dict(tileH=1, tileV=1, matchContextType=0, mapWeight=0.0, sensitivity=0.117, patchSize=9,
                              maxProbeCount=200)
    # maps: the output map rides on the target, the input map on the corpus
    small = PR.resize(img, 15, 20)
    assert small.shape == (20, 15, 3)
    rgba = np.concatenate([img, np.full((30, 40, 1), 200, np.uint8)], axis=2)
    req = PR.plugin_request(rgba, None, rgba, None, PR.PluginParameters(), map_in=img, map_out=PR.grayscale(img).repeat(3, 2))
    assert req.format == (3, 3, 1, 1, 1) and req.target.shape == (30, 40, 8)
    assert (req.target[..., 4] == 200).all() and np.array_equal(req.corpus[..., 5:], img)


@pytest.mark.parametrize("preset", ["heal", "uncrop", "fill"])
def test_preset_requests_run_on_cpu_engine(oracle, preset):
    img = _image(36, 44, 3, 7)
    if preset == "heal":
        sel = _disc(36, 44, 20, 18, 5)
        corpus, csel, p = PR.heal_selection_request(img, sel, sampling_radius=8, direction=0, order=1)
        req = PR.plugin_request(img, sel, corpus, csel, p)
    elif preset == "uncrop":
        canvas, tsel, corpus, csel, p = PR.uncrop_request(img[:24, :30], percent=20)
        req = PR.plugin_request(canvas, tsel, corpus, csel, p)
    else:
        sel = _disc(36, 44, 22, 18, 7)
        req = PR.plugin_request(img, sel, _image(16, 16, 3, 9), None, PR.PluginParameters(0, 0, 0, 0.0, 0.05, 8, 300))
    rc, out, _ = oracle.engine(make_params(**req.params), oracle.format_indices(*req.format), req.target, req.corpus)
    assert rc == 0
    sel = req.target[..., 0] != 0
    assert (out[~sel] == req.target[~sel]).all() and not (out[sel][:, 1:4] == req.target[sel][:, 1:4]).all()
