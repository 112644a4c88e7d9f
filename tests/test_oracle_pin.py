"""Pins the CPU oracle (oracle/resynth_oracle.c) to the reference engine
compiled from its own sources (oracle/build_ref.sh): every case must be
byte-identical.  Runs on CPU; skipped where the reference tree is absent."""
import numpy as np
import pytest

from oracle import make_params
from resynthesizer_gb300 import workloads as W


def P(**kw):
    d = dict(kw)
    if "sensitivity" in d:
        d["sensitivity"] = d.pop("sensitivity")
    return make_params(**d)


@pytest.mark.parametrize("sens,mw", [(0.117, 0.5), (0.05, 1.0), (0.3, 0.0), (0.117, 0.117), (1.0, 3.7)])
def test_metric_tables(oracle, reference, sens, mw):
    a, b = oracle.metric_tables(sens, mw), reference.metric_tables(sens, mw)
    assert (a[0] == b[0]).all() and (a[1] == b[1]).all()


@pytest.mark.parametrize("dims", [(1, 1, 1, 1), (5, 7, 9, 3), (40, 30, 20, 50), (64, 17, 33, 90)])
def test_sorted_offsets(oracle, reference, dims):
    assert (oracle.sorted_offsets(*dims) == reference.sorted_offsets(*dims)).all()


@pytest.mark.parametrize("ctype", range(9))
def test_target_order(oracle, reference, ctype):
    rng = W.SplitMix64(77)
    mask = W.ellipse_mask(37, 45, rng, 3, 4, 12, 0.1, 0.5)
    img = W.value_noise(37, 45, 3, rng)
    tgt, _ = W.simple_to_pixmaps(img, mask)
    fmt = oracle.format_from_type(W.T_RGB)
    rc, ref_order = reference.order_targets(P(matchContextType=ctype), fmt, tgt)
    ys, xs = np.nonzero(mask)
    mine = oracle.order_targets(ctype, np.stack([xs, ys], 1))
    assert rc == 0
    assert (mine == ref_order).all()


def test_target_order_bad_type(oracle, reference):
    tgt, _ = W.simple_to_pixmaps(np.zeros((4, 4, 3), np.uint8), np.full((4, 4), 255, np.uint8))
    rc, _ = reference.order_targets(P(matchContextType=9), oracle.format_from_type(0), tgt)
    assert rc == 4
    with pytest.raises(ValueError):
        oracle.order_targets(9, np.zeros((3, 2), np.int32))


@pytest.mark.parametrize("fmt", [W.T_RGB, W.T_RGBA, W.T_Gray, W.T_GrayA])
@pytest.mark.parametrize("ctype", [0, 1, 2, 3, 4, 5, 6, 7, 8])
def test_image_synth_formats_orders(oracle, reference, fmt, ctype):
    wl = W.heal_small(size=28, hole=9, fmt=fmt, ctype=ctype, patch=16, trys=40, index=ctype)
    p = P(**wl["params"])
    rc1, out1 = reference.image_synth(wl["image"], wl["mask"], fmt, p)
    rc2, out2, _ = oracle.image_synth(wl["image"], wl["mask"], fmt, p)
    assert rc1 == rc2 == 0
    assert (out1 == out2).all()


@pytest.mark.parametrize("patch,trys", [(0, 5), (1, 5), (2, 0), (9, 1), (64, 20)])
def test_image_synth_patch_trys(oracle, reference, patch, trys):
    wl = W.heal_small(size=24, hole=8, patch=patch, trys=trys, ctype=1)
    p = P(**wl["params"])
    rc1, out1 = reference.image_synth(wl["image"], wl["mask"], wl["fmt"], p)
    rc2, out2, _ = oracle.image_synth(wl["image"], wl["mask"], wl["fmt"], p)
    assert rc1 == rc2 == 0 and (out1 == out2).all()


def test_image_synth2_separate_corpus_mask(oracle, reference):
    wl = W.heal_small(size=26, hole=8, ctype=2)
    m2 = np.zeros_like(wl["mask"])
    m2[:, :10] = 255
    p = P(**wl["params"])
    rc1, out1 = reference.image_synth(wl["image"], wl["mask"], wl["fmt"], p, mask2=m2)
    rc2, out2, _ = oracle.image_synth(wl["image"], wl["mask"], wl["fmt"], p, mask2=m2)
    assert rc1 == rc2 == 0 and (out1 == out2).all()


def test_heal256_bit_exact(oracle, reference):
    wl = W.heal256()
    p = P(**wl["params"])
    rc1, out1 = reference.image_synth(wl["image"], wl["mask"], wl["fmt"], p)
    rc2, out2, st = oracle.image_synth(wl["image"], wl["mask"], wl["fmt"], p)
    assert rc1 == rc2 == 0 and (out1 == out2).all()
    assert st.visits == 16592 and st.passes == 6


def _engine_case(kind):
    if kind == "render_tiled":
        wl = W.render(tile=16, out=40)
        return wl, dict(wl["params"], tileH=1, tileV=1)
    if kind == "render":
        wl = W.render(tile=20, out=48)
        return wl, dict(wl["params"])
    if kind == "mapstyle":
        wl = W.mapstyle(corpus_size=24, out=40)
        return wl, dict(wl["params"])
    if kind == "mapstyle_ctx":
        wl = W.mapstyle(corpus_size=24, out=36)
        t = wl["target"].copy()
        t[:, :12, 0] = 0          # a left band of context
        t[:24, :12, 1:4] = wl["corpus"][:, :12, 1:4]
        wl = dict(wl, target=t)
        return wl, dict(wl["params"], matchContextType=3, mapWeight=1.3)
    raise KeyError(kind)


@pytest.mark.parametrize("kind", ["render_tiled", "render", "mapstyle", "mapstyle_ctx"])
def test_engine_state(oracle, reference, kind):
    wl, pk = _engine_case(kind)
    p = P(**pk)
    fmt = oracle.format_indices(*wl["format"])
    rc1, t1, s1, h1 = reference.engine_state(p, fmt, wl["target"], wl["corpus"])
    rc2, t2, _, s2, h2 = oracle.engine(p, fmt, wl["target"], wl["corpus"], want_state=True)
    assert rc1 == rc2 == 0
    assert (t1 == t2).all() and (s1 == s2).all() and (h1 == h2).all()


def _random_state(seed, tw=30, th=26, cw=22, ch=20, fmt=(3, 0, 0, 0, 0)):
    rng = np.random.default_rng(seed)
    colors, mapc = fmt[0], fmt[1]
    bpp = 1 + colors + (1 if fmt[2] or fmt[3] else 0) + (mapc if fmt[4] else 0)
    target = rng.integers(0, 256, (th, tw, bpp), dtype=np.uint8)
    corpus = rng.integers(0, 256, (ch, cw, bpp), dtype=np.uint8)
    corpus[..., 0] = np.where(rng.random((ch, cw)) < 0.85, 255, rng.integers(0, 255, (ch, cw)))
    hv = (rng.random((th, tw)) < 0.5).astype(np.uint8)
    src = np.full((th, tw, 2), -1, np.int32)
    has = rng.random((th, tw)) < 0.6
    src[has, 0] = rng.integers(-2, cw + 2, has.sum())
    src[has, 1] = rng.integers(-2, ch + 2, has.sum())
    n = 60
    targets = np.stack([rng.integers(0, tw, n), rng.integers(0, th, n)], 1).astype(np.int32)
    counts = rng.integers(0, 40, n)
    start = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    cands = np.stack([rng.integers(-3, cw + 3, start[-1]), rng.integers(-3, ch + 3, start[-1])], 1).astype(np.int32)
    return target, corpus, hv, src, targets, start, cands


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("fmt", [(3, 0, 0, 0, 0), (3, 0, 1, 1, 0), (1, 0, 0, 0, 0), (3, 1, 0, 0, 1), (1, 3, 1, 0, 1)])
def test_frozen(oracle, reference, seed, fmt):
    target, corpus, hv, src, targets, start, cands = _random_state(seed, fmt=fmt)
    f = oracle.format_indices(*fmt)
    for tiles in [(0, 0), (1, 1)]:
        p = P(patchSize=int(9 + 7 * seed), mapWeight=0.7, tileH=tiles[0], tileV=tiles[1])
        a = oracle.frozen(p, f, target, corpus, hv, src, targets, start, cands)
        b = reference.frozen(p, f, target, corpus, hv, src, targets, start, cands)
        for x, y in zip(a, b):
            assert (x == y).all()


def test_energy_matches_reference_full_sum(oracle, reference):
    target, corpus, hv, src, targets, _, _ = _random_state(5)
    f = oracle.format_indices(3, 0, 0, 0, 0)
    p = P(patchSize=30)
    tot, per = oracle.energy(p, f, target, corpus, hv, src, targets)
    sp = src[targets[:, 1], targets[:, 0]].astype(np.int32)
    start = np.arange(len(targets) + 1, dtype=np.uint32)
    ref_sum, _, _ = reference.frozen(p, f, target, corpus, hv, src, targets, start, sp, full_sum=True)
    assert (per == ref_sum).all() and tot == int(ref_sum.astype(np.uint64).sum())


def test_error_codes(oracle, reference):
    img = np.zeros((1, 3), np.uint8) + np.array([[128, 64, 1]], np.uint8)
    mask = np.array([[0, 255, 0]], np.uint8)
    for p, m, fmt, expect in [
        (P(patchSize=65), mask, W.T_Gray, 3),
        (P(), np.array([[0]], np.uint8), W.T_Gray, 2),
        (P(), np.zeros((1, 3), np.uint8), W.T_Gray, 5),
        (P(), mask, 7, 1),
        (P(matchContextType=9), mask, W.T_Gray, 4),
    ]:
        rc1, out1 = reference.image_synth(img[..., None], m, fmt, p)
        rc2, out2, _ = oracle.image_synth(img[..., None], m, fmt, p)
        assert rc1 == rc2 == expect
        assert (out1 == img[..., None]).all() and (out2 == img[..., None]).all()
    rgba = np.array([[[128, 128, 128, 0], [1, 1, 1, 1], [0, 0, 0, 0]]], np.uint8)
    rc1, _ = reference.image_synth(rgba, mask, W.T_RGBA, P())
    rc2, _, _ = oracle.image_synth(rgba, mask, W.T_RGBA, P())
    assert rc1 == rc2 == 6


def test_cancel_and_progress(oracle, reference):
    wl = W.heal_small(size=120, hole=70, ctype=1, patch=9, trys=20)
    p = P(**wl["params"])
    seen_r, seen_o = [], []
    rc1, out1 = reference.image_synth(wl["image"], wl["mask"], wl["fmt"], p, progress=lambda a, b: seen_r.append(a))
    rc2, out2, _ = oracle.image_synth(wl["image"], wl["mask"], wl["fmt"], p, progress=lambda a, b: seen_o.append(a))
    assert rc1 == rc2 == 0 and seen_r == seen_o and len(seen_r) > 3 and (out1 == out2).all()
    rc1, out1 = reference.image_synth(wl["image"], wl["mask"], wl["fmt"], p, cancel=1)
    rc2, out2, _ = oracle.image_synth(wl["image"], wl["mask"], wl["fmt"], p, cancel=1)
    assert rc1 == rc2 == 0 and (out1 == wl["image"]).all() and (out2 == wl["image"]).all()


def test_rand_stream_is_libc(oracle):
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand(1198472)
    expect = [libc.rand() for _ in range(100)]
    assert list(oracle.rand_stream(100)) == expect


def test_threaded_oracle_runs(oracle):
    wl = W.heal_small(size=40, hole=14, ctype=2)
    p = P(**wl["params"])
    rc, out, st = oracle.image_synth(wl["image"], wl["mask"], wl["fmt"], p, threads=8)
    assert rc == 0 and st.visits >= 14 * 14 * 2
    assert (out[wl["mask"] == 0] == wl["image"][wl["mask"] == 0]).all()
