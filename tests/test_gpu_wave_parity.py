"""Wavefront mode against its CPU restatement, through every entry a caller
uses: the Simple API (imageSynth / imageSynth2, whose adaption and write-back
run on the device for random orders and on the host otherwise), the
many-request entry imageSynthBatch (its shared many-request launches), every
visit order (matchContextType 0..8, the directional and brushfire orders in
the reference's own order) and degenerate shapes.  The oracle is
oracle/wave_oracle.c behind the reference's Simple-API adapters
(oracle/resynth_oracle.c, simple_api); every comparison is byte for byte."""
import numpy as np
import pytest

import resynthesizer_gb300 as R
from oracle import make_params
from resynthesizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu

WAVE = dict(mode=R.MODE_WAVEFRONT)
FORMATS = [W.T_RGB, W.T_RGBA, W.T_Gray, W.T_GrayA]


@pytest.fixture(scope="module", autouse=True)
def built():
    from resynthesizer_gb300 import build
    build.build()
    R.lib()


def _with_transparency(img, fmt, seed):
    """Alpha formats: about a tenth of the pixels fully transparent (neither
    context nor corpus, lib/engine.c:338-431)."""
    if fmt not in (W.T_RGBA, W.T_GrayA):
        return img
    img = img.copy()
    rng = np.random.default_rng(seed)
    img[..., -1] = np.where(rng.random(img.shape[:2]) < 0.1, 0, 255)
    return img


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("ctype", range(9))
def test_simple_api_wavefront_vs_oracle(oracle, fmt, ctype):
    """imageSynth in wavefront mode, every layout and every visit order, on
    row-padded caller buffers: byte-identical to the restatement."""
    wl = W.heal_small(size=40, hole=15, fmt=fmt, ctype=ctype, patch=16 if ctype % 2 else 25, trys=60,
                      index=7 + ctype)
    img = _with_transparency(wl["image"], fmt, 100 * fmt + ctype)
    r = R.image_synth(img, wl["mask"], fmt, R.params(**wl["params"]), opts=R.options(**WAVE), row_pad=3 + ctype)
    rc, out = oracle.wave_image_synth(img, wl["mask"], fmt, make_params(**wl["params"]))
    assert r.rc == rc == 0, R.last_error()
    assert np.array_equal(r.out, out)


@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("ctype", [1, 2])
def test_simple_api2_wavefront_vs_oracle(oracle, fmt, ctype):
    """imageSynth2: the corpus is the second mask (here a ring around the
    hole), not the inverted first one."""
    wl = W.heal_small(size=44, hole=14, fmt=fmt, ctype=ctype, patch=20, trys=50, index=31 + ctype)
    img = _with_transparency(wl["image"], fmt, 7 * fmt + ctype)
    mask2 = np.zeros_like(wl["mask"])
    mask2[6:38, 6:38] = 255
    mask2[wl["mask"] != 0] = 0
    r = R.image_synth(img, wl["mask"], fmt, R.params(**wl["params"]), mask2=mask2, opts=R.options(**WAVE),
                      row_pad=5)
    rc, out = oracle.wave_image_synth(img, wl["mask"], fmt, make_params(**wl["params"]), mask2=mask2)
    assert r.rc == rc == 0, R.last_error()
    assert np.array_equal(r.out, out)


@pytest.mark.parametrize("ctype", range(2, 9))
def test_engine_directional_orders_vs_oracle(oracle, ctype):
    """engine() on pixmaps with the directional and brushfire orders (types
    2..8, the reference's own visit order cut into bands): a larger heal so
    that pass 0 has several bands, plus map channels and tiling on two of
    them."""
    if ctype in (4, 7):
        wl = W.mapstyle(corpus_size=40, out=72, index=ctype)
        kw = dict(wl["params"], matchContextType=ctype, tileH=int(ctype == 7), tileV=int(ctype == 7))
        t, c, spec = wl["target"], wl["corpus"], wl["format"]
    else:
        wl = W.heal_small(size=120, hole=70, ctype=ctype, patch=30, trys=80, index=50 + ctype)
        t, c = W.simple_to_pixmaps(wl["image"], wl["mask"])
        spec, kw = (3, 0, 0, 0, 0), wl["params"]
    r = R.engine(t, c, R.format_indices(*spec), R.params(**kw), opts=R.options(**WAVE))
    rc, out, passes, betters = oracle.wave_engine(make_params(**kw), oracle.format_indices(*spec), t, c)
    assert r.rc == 0 == rc, R.last_error()
    assert r.stats["passes"] == passes and list(r.stats["betters"])[:passes] == betters
    assert np.array_equal(r.out, out)


def test_batch_requests_vs_oracle(oracle):
    """imageSynthBatch on a mix like the many-request workload: Gray, RGB and
    RGBA requests of uneven sizes, patch sizes 9, 16 and 30, holes of 2-20 %,
    requests that stop after different numbers of passes.  Every request's
    output equals the restatement's, byte for byte."""
    reqs = W.batch_requests(n=18, lo=40, hi=140, index=23)
    items = [(r["image"], r["mask"], r["fmt"], R.params(**r["params"])) for r in reqs]
    assert {r["fmt"] for r in reqs} == {W.T_Gray, W.T_RGB, W.T_RGBA}
    assert {r["params"]["patchSize"] for r in reqs} == {9, 16, 30}
    rc, outs, codes, st = R.image_synth_batch(items, opts=R.options(**WAVE), concurrency=4)
    assert rc == 0 and codes == [0] * len(reqs), R.last_error()
    for i, (r, out) in enumerate(zip(reqs, outs)):
        rc_o, out_o = oracle.wave_image_synth(r["image"], r["mask"], r["fmt"], make_params(**r["params"]))
        assert rc_o == 0
        assert np.array_equal(out, out_o), i


def test_batch_transparent_and_mixed_orders_vs_oracle(oracle):
    """A batch whose requests carry transparent pixels and mix random orders
    (shared launches) with directional ones (host workers)."""
    reqs = W.batch_requests(n=8, lo=48, hi=96, index=29)
    items = []
    for i, r in enumerate(reqs):
        img = _with_transparency(r["image"], r["fmt"], 1000 + i)
        kw = dict(r["params"], matchContextType=[1, 0, 2, 1, 5, 1, 8, 0][i])
        items.append((img, r["mask"], r["fmt"], kw))
    rc, outs, codes, _ = R.image_synth_batch([(a, b, c, R.params(**d)) for a, b, c, d in items],
                                             opts=R.options(**WAVE), concurrency=3)
    assert rc == 0 and codes == [0] * len(items), R.last_error()
    for i, ((img, mask, fmt, kw), out) in enumerate(zip(items, outs)):
        rc_o, out_o = oracle.wave_image_synth(img, mask, fmt, make_params(**kw))
        assert rc_o == 0 and np.array_equal(out, out_o), i


EDGE = ["1x3", "3x3_p0", "5x4_p1", "7x7_p2", "9x6_p64", "tiny_corpus", "tiled_8x8", "gray_alpha", "row_16x1"]


def edge_case(case):
    """(image, mask, format, params) of a tiny or degenerate problem."""
    rng = np.random.default_rng(len(case))
    fmt = W.T_RGB
    patch, tile = 16, (0, 0)
    if case == "1x3":
        img = rng.integers(0, 256, (1, 3, 3), dtype=np.uint8)
        mask = np.array([[0, 255, 0]], np.uint8)
    elif case == "row_16x1":
        img = rng.integers(0, 256, (1, 16, 3), dtype=np.uint8)
        mask = np.zeros((1, 16), np.uint8)
        mask[0, 5:11] = 255
    elif case == "tiny_corpus":
        img = rng.integers(0, 256, (6, 6, 3), dtype=np.uint8)
        mask = np.full((6, 6), 255, np.uint8)
        mask[0, 0] = 0                      # a single corpus pixel
    elif case == "gray_alpha":
        fmt = W.T_GrayA
        img = rng.integers(0, 256, (12, 10, 2), dtype=np.uint8)
        img[..., 1] = 255
        mask = np.zeros((12, 10), np.uint8)
        mask[3:8, 2:7] = 255
    else:
        h, w = {"3x3_p0": (3, 3), "5x4_p1": (5, 4), "7x7_p2": (7, 7), "9x6_p64": (9, 6), "tiled_8x8": (8, 8)}[case]
        patch = {"3x3_p0": 0, "5x4_p1": 1, "7x7_p2": 2, "9x6_p64": 64, "tiled_8x8": 9}[case]
        if case == "tiled_8x8":
            tile = (1, 1)
        img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
        mask = np.zeros((h, w), np.uint8)
        mask[h // 3:h - h // 3, w // 3:w - w // 3] = 255
    kw = dict(tileH=tile[0], tileV=tile[1], matchContextType=1, patchSize=patch, maxProbeCount=50)
    return img, mask, fmt, kw


@pytest.mark.parametrize("case", EDGE)
def test_wavefront_edge_cases_vs_oracle(oracle, case):
    """The degenerate shapes through engine() and through the Simple API,
    each against the restatement."""
    img, mask, fmt, kw = edge_case(case)
    tgt, cor = W.simple_to_pixmaps(img, mask)
    spec = {W.T_RGB: (3, 0, 0, 0, 0), W.T_GrayA: (1, 0, 1, 1, 0)}[fmt]
    r = R.engine(tgt, cor, R.format_indices(*spec), R.params(**kw), opts=R.options(**WAVE))
    rc, out, passes, betters = oracle.wave_engine(make_params(**kw), oracle.format_indices(*spec), tgt, cor)
    assert r.rc == 0 == rc, R.last_error()
    assert r.stats["passes"] == passes and list(r.stats["betters"])[:passes] == betters
    assert np.array_equal(r.out, out)
    s = R.image_synth(img, mask, fmt, R.params(**kw), opts=R.options(**WAVE))
    rc_o, out_o = oracle.wave_image_synth(img, mask, fmt, make_params(**kw))
    assert s.rc == rc_o == 0 and np.array_equal(s.out, out_o)


def test_batch_more_requests_than_one_launch_takes(oracle):
    """More requests than one persistent many-request launch takes (4096):
    the pass is split into launches of at most 4096 requests.  4,300 tiny
    heals of mixed layouts, each byte-identical to the restatement."""
    rng = np.random.default_rng(41)
    items = []
    for i in range(4300):
        fmt = [W.T_Gray, W.T_RGB, W.T_RGBA][i % 3]
        h, w = int(rng.integers(6, 14)), int(rng.integers(6, 14))
        img = rng.integers(0, 256, (h, w, W.PIXELELS[fmt]), dtype=np.uint8)
        if fmt == W.T_RGBA:
            img[..., 3] = 255
        mask = np.zeros((h, w), np.uint8)
        y0, x0 = int(rng.integers(1, h - 3)), int(rng.integers(1, w - 3))
        mask[y0:y0 + 2, x0:x0 + 3] = 255
        kw = dict(matchContextType=1, patchSize=[9, 16, 30][i % 3], maxProbeCount=20)
        items.append((img, mask, fmt, kw))
    rc, outs, codes, st = R.image_synth_batch([(a, b, c, R.params(**d)) for a, b, c, d in items],
                                              opts=R.options(**WAVE), concurrency=4)
    assert rc == 0 and codes == [0] * len(items), R.last_error()
    for i, ((img, mask, fmt, kw), out) in enumerate(zip(items, outs)):
        rc_o, out_o = oracle.wave_image_synth(img, mask, fmt, make_params(**kw), threads=1)
        assert rc_o == 0 and np.array_equal(out, out_o), i
