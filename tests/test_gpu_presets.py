"""Plug-in presets through the GPU engine: in replay mode each preset's
request gives exactly the CPU engine's output (same request, same
reference semantics); in wavefront mode the invariants hold."""
import numpy as np
import pytest

import resynthesizer_gb300 as R
from oracle import make_params
from resynthesizer_gb300 import presets as PR
from resynthesizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from resynthesizer_gb300 import build
    build.build()
    R.lib()


def _image(h, w, c, seed):
    return W.value_noise(h, w, c, W.SplitMix64(seed))


def _disc(h, w, cx, cy, r):
    y, x = np.mgrid[0:h, 0:w]
    return (x - cx) ** 2 + (y - cy) ** 2 <= r * r


def _requests():
    img = _image(40, 48, 3, 11)
    sel = _disc(40, 48, 22, 20, 6)
    out = {}
    for d, o in [(0, 0), (1, 1), (2, 2)]:
        corpus, csel, p = PR.heal_selection_request(img, sel, sampling_radius=9, direction=d, order=o)
        out[f"heal_d{d}_o{o}"] = PR.plugin_request(img, sel, corpus, csel, p)
    canvas, tsel, corpus, csel, p = PR.uncrop_request(img[:30, :36], percent=20)
    out["uncrop"] = PR.plugin_request(canvas, tsel, corpus, csel, p)
    out["render_tile"] = PR.plugin_request(np.full((40, 40, 3), 255, np.uint8), None, img[:20, :20], None,
                                           PR.PluginParameters(1, 1, 0, 0.0, 0.117, 9, 200))
    out["fill"] = PR.plugin_request(img, sel, _image(16, 16, 3, 12), None, PR.PluginParameters(0, 0, 0, 0.0, 0.05, 8, 300))
    small = PR.resize(img, 24, 20)
    out["enlarge"] = PR.plugin_request(PR.resize(small, 48, 40), None, small, None,
                                       PR.PluginParameters(0, 0, 0, 1.0, 0.117, 8, 500),
                                       map_in=PR.resize(PR.resize(small, 12, 10), 24, 20), map_out=PR.resize(small, 48, 40))
    style = _image(24, 24, 3, 13)
    out["map_style"] = PR.plugin_request(img, None, style, None,
                                         PR.PluginParameters(1, 1, 1, PR.map_weight_for_transfer(10), 0.117, 9, 200),
                                         map_in=PR.grayscale(style), map_out=PR.grayscale(img))
    return out


REQS = _requests()


@pytest.mark.parametrize("name", sorted(REQS))
def test_preset_replay_matches_cpu_engine(oracle, name):
    req = REQS[name]
    g = PR.run_request(req, opts=R.options(mode=R.MODE_REPLAY))
    rc, out, _ = oracle.engine(make_params(**req.params), oracle.format_indices(*req.format), req.target, req.corpus)
    assert g.rc == rc == 0 and np.array_equal(g.out, out)


@pytest.mark.parametrize("name", sorted(REQS))
def test_preset_wavefront_invariants(name):
    req = REQS[name]
    r = PR.run_request(req, opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1))
    assert r.rc == 0
    sel = req.target[..., 0] != 0
    assert (r.out[~sel] == req.target[~sel]).all()
    src = r.source[sel]
    assert (src[:, 0] >= 0).all()
    nc = req.format[0]
    assert (r.out[sel][:, 1:1 + nc] == req.corpus[src[:, 1], src[:, 0], 1:1 + nc]).all()
    # every source is a corpus pixel that was selected
    assert (req.corpus[src[:, 1], src[:, 0], 0] == 255).all()


def test_preset_functions_return_images():
    img = _image(40, 48, 3, 21)
    sel = _disc(40, 48, 24, 20, 5)
    rc, out, _ = PR.heal_selection(img, sel, sampling_radius=10)
    assert rc == 0 and out.shape == img.shape and (out[~sel] == img[~sel]).all()
    rc, out, _ = PR.uncrop(img, percent=10)
    assert rc == 0 and out.shape == (44, 52, 3)
    rc, out, _ = PR.render_texture(img, resize_ratio=1.5, make_tile=True)
    assert rc == 0 and out.shape == (60, 72, 3)
    rgba = np.concatenate([img, np.full((40, 48, 1), 255, np.uint8)], axis=2)
    rgba[10:15, 10:20, 3] = 0
    rc, out, _ = PR.heal_transparency(rgba, sampling_radius=8)
    assert rc == 0 and out.shape == (40, 48, 3)
    rc, out, _ = PR.sharpen(img, 2.0)
    assert rc == 0 and out.shape == img.shape
    rc, out, _ = PR.enlarge(img[:20, :24], 2.0)
    assert rc == 0 and out.shape == (40, 48, 3)
    rc, out, _ = PR.map_style(img, _image(24, 24, 3, 22), percent_transfer=30, map_by_brightness=True)
    assert rc == 0 and out.shape == img.shape
