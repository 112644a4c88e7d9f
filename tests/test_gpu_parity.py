"""GPU parity: the CUDA engine through the C ABI against the golden fixtures
(made by the reference engine) and against the CPU oracle on the same seeded
inputs.  Integer work throughout, so every comparison is exact unless it is a
wavefront-mode quality bound (stated per test)."""
import hashlib

import numpy as np
import pytest

import golden_cases as G
import resynthesizer_gb300 as R
from oracle import make_params
from resynthesizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from resynthesizer_gb300 import build
    build.build()
    R.lib()


def rp(d):
    return R.params(**d) if d is not None else None


def op(d):
    return make_params(**d)


REPLAY = dict(mode=R.MODE_REPLAY)

# ------------------------------------------------------------ frozen state


@pytest.mark.parametrize("k", range(4))
def test_frozen_golden(k):
    c = G.frozen()[k]
    fmt = R.format_indices(*c["format"])
    s, pt, cnt = R.frozen_best_fit(rp(c["params"]), fmt, c["target"], c["corpus"], c["has"], c["source"],
                                   c["targets"], c["start"], c["cands"])
    assert (cnt == c["count"]).all()
    assert (s == c["sum"]).all()
    assert (pt == c["pt"]).all()


def _random_state(seed, fmt, tw=70, th=50, cw=40, ch=36, ncand=300):
    rng = np.random.default_rng(seed)
    bpp = 1 + fmt[0] + (1 if fmt[2] or fmt[3] else 0) + (fmt[1] if fmt[4] else 0)
    target = rng.integers(0, 256, (th, tw, bpp), dtype=np.uint8)
    corpus = rng.integers(0, 256, (ch, cw, bpp), dtype=np.uint8)
    corpus[..., 0] = np.where(rng.random((ch, cw)) < 0.9, 255, rng.integers(0, 255, (ch, cw)))
    hv = (rng.random((th, tw)) < rng.uniform(0.05, 0.9)).astype(np.uint8)
    src = np.full((th, tw, 2), -1, np.int32)
    has = rng.random((th, tw)) < 0.6
    src[has, 0] = rng.integers(0, cw, has.sum())
    src[has, 1] = rng.integers(0, ch, has.sum())
    n = 400
    targets = np.stack([rng.integers(0, tw, n), rng.integers(0, th, n)], 1).astype(np.int32)
    counts = rng.integers(0, ncand, n)
    start = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint32)
    cands = np.stack([rng.integers(-3, cw + 3, start[-1]), rng.integers(-3, ch + 3, start[-1])], 1).astype(np.int32)
    # repeat some candidates so ties in the sum must be broken by list order
    cands[1::7] = cands[0::7][: len(cands[1::7])]
    return target, corpus, hv, src, targets, start, cands


@pytest.mark.parametrize("seed", [11, 12])
@pytest.mark.parametrize("fmt", [(3, 0, 0, 0, 0), (3, 0, 1, 1, 0), (1, 0, 0, 0, 0), (3, 1, 0, 0, 1),
                                 (1, 3, 1, 0, 1), (2, 2, 0, 1, 1)])
@pytest.mark.parametrize("patch", [1, 9, 30, 64])
def test_frozen_vs_oracle(oracle, seed, fmt, patch):
    target, corpus, hv, src, targets, start, cands = _random_state(seed + patch, fmt)
    for tile in (0, 1):
        kw = dict(patchSize=patch, mapWeight=0.37 * seed, tileH=tile, tileV=tile)
        f = R.format_indices(*fmt)
        a = R.frozen_best_fit(R.params(**kw), f, target, corpus, hv, src, targets, start, cands)
        b = oracle.frozen(op(kw), oracle.format_indices(*fmt), target, corpus, hv, src, targets, start, cands)
        for x, y in zip(a, b):
            assert (x == y).all()


@pytest.mark.parametrize("fmt", [(3, 0, 0, 0, 0), (3, 1, 0, 0, 1)])
def test_energy_vs_oracle(oracle, fmt):
    target, corpus, hv, src, targets, _, _ = _random_state(5, fmt)
    kw = dict(patchSize=30, mapWeight=0.9)
    e1, per1 = R.patch_energy(R.params(**kw), R.format_indices(*fmt), target, corpus, hv, src, targets)
    e2, per2 = oracle.energy(op(kw), oracle.format_indices(*fmt), target, corpus, hv, src, targets)
    assert e1 == e2 and (per1 == per2).all()

# ------------------------------------------------------------ replay mode


def test_replay_testsynth_known_answers():
    for c in G.testsynth():
        r = R.image_synth(c["image"], c["mask"], c["fmt"], rp(c["params"]), opts=R.options(**REPLAY))
        assert r.rc == c["rc"], c["name"]
        assert (r.out == c["out"]).all(), c["name"]


@pytest.mark.parametrize("k", range(16))
def test_replay_golden_heal(k):
    c = G.heal()[k]
    r = R.image_synth(c["image"], c["mask"], c["fmt"], rp(c["params"]), opts=R.options(**REPLAY))
    assert r.rc == 0 and (r.out == c["out"]).all()


def test_replay_heal256_bit_exact():
    c = G.heal256()
    r = R.image_synth(c["image"], c["mask"], c["fmt"], rp(c["params"]), opts=R.options(**REPLAY))
    assert r.rc == 0
    assert (r.out[96:160, 96:160] == c["out_region"]).all()
    assert hashlib.sha256(r.out.tobytes()).hexdigest() == c["sha256"]
    assert r.stats["visits"] == 16592 and r.stats["passes"] == 6


def test_replay_golden_engine_state():
    for c in G.engine():
        fmt = R.format_indices(*c["format"])
        r = R.engine(c["target"], c["corpus"], fmt, rp(c["params"]), opts=R.options(recordState=1, **REPLAY))
        assert r.rc == 0, c["name"]
        assert (r.out == c["out"]).all(), c["name"]
        assert (r.source == c["source"]).all() and (r.has_value == c["has"]).all(), c["name"]


@pytest.mark.parametrize("fmt", [W.T_RGB, W.T_RGBA, W.T_Gray, W.T_GrayA])
@pytest.mark.parametrize("ctype", [0, 3, 4, 6, 7])
def test_replay_vs_oracle_orders(oracle, fmt, ctype):
    wl = W.heal_small(size=36, hole=13, fmt=fmt, ctype=ctype, patch=25, trys=60, index=3 + ctype)
    r = R.image_synth(wl["image"], wl["mask"], fmt, rp(wl["params"]), opts=R.options(**REPLAY))
    rc, out, st = oracle.image_synth(wl["image"], wl["mask"], fmt, op(wl["params"]))
    assert r.rc == rc == 0 and (r.out == out).all()
    assert r.stats["evals"] == st.evals


@pytest.mark.parametrize("patch,trys", [(0, 3), (2, 0), (64, 300), (16, 1)])
def test_replay_vs_oracle_edges(oracle, patch, trys):
    wl = W.heal_small(size=30, hole=10, patch=patch, trys=trys, ctype=1, index=patch)
    r = R.image_synth(wl["image"], wl["mask"], wl["fmt"], rp(wl["params"]), opts=R.options(**REPLAY))
    rc, out, _ = oracle.image_synth(wl["image"], wl["mask"], wl["fmt"], op(wl["params"]))
    assert r.rc == rc == 0 and (r.out == out).all()


def test_replay_engine_tiled_maps_vs_oracle(oracle):
    wl = W.mapstyle(corpus_size=32, out=48, index=2)
    kw = dict(wl["params"], tileH=1, tileV=0, mapWeight=0.8)
    fmt = R.format_indices(*wl["format"])
    r = R.engine(wl["target"], wl["corpus"], fmt, R.params(**kw), opts=R.options(recordState=1, **REPLAY))
    rc, out, _, src, hv = oracle.engine(op(kw), oracle.format_indices(*wl["format"]), wl["target"], wl["corpus"],
                                        want_state=True)
    assert r.rc == rc == 0 and (r.out == out).all() and (r.source == src).all() and (r.has_value == hv).all()


def test_replay_progress_and_cancel(oracle):
    wl = W.heal_small(size=120, hole=70, ctype=1, patch=9, trys=20)
    seen_g, seen_o = [], []
    r = R.image_synth(wl["image"], wl["mask"], wl["fmt"], rp(wl["params"]), opts=R.options(**REPLAY),
                      progress=lambda a, b: seen_g.append(a))
    rc, out, _ = oracle.image_synth(wl["image"], wl["mask"], wl["fmt"], op(wl["params"]),
                                    progress=lambda a, b: seen_o.append(a))
    assert r.rc == rc == 0 and seen_g == seen_o and (r.out == out).all()
    for mode in (R.MODE_REPLAY, R.MODE_WAVEFRONT):
        r = R.image_synth(wl["image"], wl["mask"], wl["fmt"], rp(wl["params"]), opts=R.options(mode=mode), cancel=1)
        assert r.rc == 0 and (r.out == wl["image"]).all()


def test_reference_entry_points_use_selected_mode():
    c = G.heal()[0]
    prev = R.lib().resynthSetMode(R.MODE_REPLAY)
    try:
        r = R.image_synth(c["image"], c["mask"], c["fmt"], rp(c["params"]), raw_entry=True)
    finally:
        R.lib().resynthSetMode(prev)
    assert r.rc == 0 and (r.out == c["out"]).all()

# --------------------------------------------------------- wavefront mode


@pytest.mark.parametrize("name", ["render1024", "heal4096", "mapstyle2048"])
def test_wavefront_bit_exact_full_size(name):
    """The default mode on the full-size workloads gives exactly the output of
    its CPU restatement (oracle/wave_oracle.c; hashes pinned in
    golden_cases.WAVE_FULL and checked against the oracle by
    tests/test_wave_oracle.py)."""
    t, c, spec, kw = G.wave_workload(name)
    r = R.engine(t, c, R.format_indices(*spec), R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT))
    sha, npass, nbetter = G.WAVE_FULL[name]
    assert r.rc == 0
    assert r.stats["passes"] == npass and list(r.stats["betters"])[:npass] == nbetter
    assert hashlib.sha256(r.out.tobytes()).hexdigest() == sha


@pytest.mark.parametrize("case", ["heal", "render", "render_tiled", "mapstyle"])
def test_wavefront_bit_exact_vs_wave_oracle(oracle, case):
    """Small problems (corpus staged in shared memory, teams of warps per
    target, tiling) against the CPU restatement of the wavefront mode."""
    t, c, spec, kw = G.wave_small_case(case)
    r = R.engine(t, c, R.format_indices(*spec), R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT))
    rc, out, passes, betters = oracle.wave_engine(make_params(**kw), oracle.format_indices(*spec), t, c)
    assert r.rc == 0 == rc
    assert r.stats["passes"] == passes and list(r.stats["betters"])[:passes] == betters
    assert np.array_equal(r.out, out)


@pytest.mark.parametrize("patch", [1, 2, 33, 64])
@pytest.mark.parametrize("case", ["heal", "render"])
def test_wavefront_patch_limits_vs_wave_oracle(oracle, case, patch):
    """The pass-0 nearest-key lists at their limits -- one entry, 32 and 33
    (both register halves), 63 -- on the cell-grid path (heal) and the
    valued-list path with team merges (render) against the restatement."""
    t, c, spec, kw = G.wave_small_case(case)
    kw = dict(kw, patchSize=patch)
    r = R.engine(t, c, R.format_indices(*spec), R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT))
    rc, out, passes, betters = oracle.wave_engine(make_params(**kw), oracle.format_indices(*spec), t, c)
    assert r.rc == 0 == rc
    assert r.stats["passes"] == passes and list(r.stats["betters"])[:passes] == betters
    assert np.array_equal(r.out, out)


@pytest.mark.parametrize("case", ["heal", "render", "mapstyle"])
def test_wavefront_invariants_and_energy(oracle, case):
    if case == "heal":
        wl = W.heal_small(size=96, hole=40, ctype=2, patch=30, trys=200)
        tgt, cor = W.simple_to_pixmaps(wl["image"], wl["mask"])
        spec = (3, 0, 0, 0, 0)
        kw = wl["params"]
    elif case == "render":
        wl = W.render(tile=48, out=96)
        tgt, cor, spec, kw = wl["target"], wl["corpus"], wl["format"], wl["params"]
    else:
        wl = W.mapstyle(corpus_size=48, out=96)
        tgt, cor, spec, kw = wl["target"], wl["corpus"], wl["format"], wl["params"]
    fmt = R.format_indices(*spec)
    r = R.engine(tgt, cor, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1))
    assert r.rc == 0
    sel = tgt[..., 0] != 0
    # untouched: every non-target pixel, and the mask/alpha/map bytes everywhere
    assert (r.out[~sel] == tgt[~sel]).all()
    assert (r.out[..., 0] == tgt[..., 0]).all() and (r.out[..., fmt.colorEndBip:] == tgt[..., fmt.colorEndBip:]).all()
    # every target pixel got a source whose colour it carries
    src = r.source[sel]
    assert (src[:, 0] >= 0).all() and r.has_value[sel].all()
    nc = fmt.img_match_bpp
    assert (r.out[sel][:, 1:1 + nc] == cor[src[:, 1], src[:, 0], 1:1 + nc]).all()
    # energy against the single-threaded oracle run on the same input.  At
    # these small sizes the reference's own threaded engine lands 5-16% above
    # its single-threaded result (render 96x96: +14..16%), so the bound here is
    # 25%; the 1% gate against the threaded reference is taken at full size.
    ys, xs = np.nonzero(sel)
    targets = np.stack([xs, ys], 1).astype(np.int32)
    e_gpu, _ = R.patch_energy(R.params(**kw), fmt, r.out, cor, r.has_value, r.source, targets)
    rc, out_o, _, src_o, hv_o = oracle.engine(op(kw), oracle.format_indices(*spec), tgt, cor, want_state=True)
    e_ref, _ = R.patch_energy(R.params(**kw), fmt, out_o, cor, hv_o, src_o, targets)
    assert e_gpu <= 1.25 * e_ref, (e_gpu, e_ref)


@pytest.mark.parametrize("out", [80, 300])
def test_wavefront_deterministic(out):
    # Near the image border a refinement-pass patch reaches past the colour
    # phase spacing: the result must still not depend on the order in which
    # the targets of one batch run.
    wl = W.render(tile=32, out=out)
    fmt = R.format_indices(*wl["format"])
    runs = [R.engine(wl["target"], wl["corpus"], fmt, R.params(**wl["params"]),
                     opts=R.options(mode=R.MODE_WAVEFRONT, warpsPerBlock=w)) for w in (16, 16, 8, 4)]
    assert all(r.rc == 0 for r in runs)
    assert all((r.out == runs[0].out).all() for r in runs[1:])


@pytest.mark.parametrize("density", [0.0005, 0.01, 0.2])
def test_cell_grid_patches_equal_offset_walk(density):
    # the pass-0 patch builder for far-reaching patches (cell grid) against
    # the offset-list walk, over sparse value maps and targets deep in holes
    rng = np.random.default_rng(int(density * 1e4))
    h, w = 300, 420
    hv = (rng.random((h, w)) < density).astype(np.uint8)
    hv[100:260, 50:300] = 0                      # a large hole
    ys, xs = np.nonzero(hv == 0)
    pick = rng.choice(len(xs), 300, replace=False)
    targets = np.stack([xs[pick], ys[pick]], 1)
    for p in (1, 2, 9, 16, 30, 33, 34, 64):   # list limits 1 .. 63, both register halves
        a = R.patch_neighbours(hv, p, targets, use_grid=False)
        b = R.patch_neighbours(hv, p, targets, use_grid=True)
        for i in range(len(targets)):
            assert np.array_equal(a[i], b[i]), (p, i)


@pytest.mark.parametrize("case", ["render", "heal"])
def test_wavefront_graphs_identical(case):
    # each pass launched as one captured CUDA graph gives the same output
    if case == "render":
        wl = W.render(tile=32, out=160)
        tgt, cor, spec, kw = wl["target"], wl["corpus"], wl["format"], wl["params"]
    else:
        wl = W.heal4096(index=1, size=256)
        tgt, cor = W.simple_to_pixmaps(wl["image"], wl["mask"])
        spec, kw = (3, 0, 0, 0, 0), wl["params"]
    fmt = R.format_indices(*spec)
    a = R.engine(tgt, cor, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT, warpsPerBlock=16))
    b = R.engine(tgt, cor, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT, warpsPerBlock=16, graphs=1))
    assert a.rc == b.rc == 0 and (a.out == b.out).all()


def test_batch_matches_single_calls(oracle):
    # more than 16 distinct sizes across 4 workers: shared host caches get evicted while in use
    reqs = W.batch_requests(n=24, lo=40, hi=120, index=5)
    items = [(r["image"], r["mask"], r["fmt"], R.params(**r["params"])) for r in reqs]
    rc, outs, codes, st = R.image_synth_batch(items, opts=R.options(mode=R.MODE_WAVEFRONT), concurrency=4)
    assert rc == 0 and codes == [0] * len(reqs)
    for r, out in zip(reqs, outs):
        single = R.image_synth(r["image"], r["mask"], r["fmt"], R.params(**r["params"]),
                               opts=R.options(mode=R.MODE_WAVEFRONT))
        assert single.rc == 0 and (single.out == out).all()
    # one stream per request, and the many-request path with one launch per
    # step instead of one persistent launch per pass, give the same results
    rc2, outs2, codes2, st2 = R.image_synth_batch(items, opts=R.options(mode=R.MODE_WAVEFRONT, separateRequests=1),
                                                  concurrency=4)
    assert rc2 == 0 and all((a == b).all() for a, b in zip(outs, outs2))
    rc3, outs3, codes3, st3 = R.image_synth_batch(items, opts=R.options(mode=R.MODE_WAVEFRONT, batchLaunches=1),
                                                  concurrency=4)
    assert rc3 == 0 and all((a == b).all() for a, b in zip(outs, outs3))
    assert st["launches"] < st3["launches"] / 2
    # replay mode through the batch entry point is still byte-identical to the oracle
    rc, outs, codes, _ = R.image_synth_batch(items[:2], opts=R.options(mode=R.MODE_REPLAY), concurrency=2)
    assert rc == 0
    for r, out in zip(reqs[:2], outs):
        rc_o, out_o, _ = oracle.image_synth(r["image"], r["mask"], r["fmt"], op(r["params"]))
        assert rc_o == 0 and (out_o == out).all()


@pytest.mark.parametrize("case", ["1x3", "3x3_p0", "5x4_p1", "7x7_p2", "9x6_p64", "tiny_corpus", "tiled_8x8",
                                  "gray_alpha", "row_16x1"])
def test_wavefront_edge_cases(case):
    """Tiny and degenerate problems in wavefront mode: every target gets a
    source whose colour it carries; the rest of the image is untouched."""
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
    tgt, cor = W.simple_to_pixmaps(img, mask)
    nb = img.shape[2]
    f = R.format_indices(*{W.T_RGB: (3, 0, 0, 0, 0), W.T_GrayA: (1, 0, 1, 1, 0)}[fmt])
    r = R.engine(tgt, cor, f, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1))
    assert r.rc == 0, R.last_error()
    sel = mask != 0
    assert (r.out[~sel] == tgt[~sel]).all()
    src = r.source[sel]
    assert (src[:, 0] >= 0).all()
    nc = f.img_match_bpp
    assert (r.out[sel][:, 1:1 + nc] == cor[src[:, 1], src[:, 0], 1:1 + nc]).all()
    assert (cor[src[:, 1], src[:, 0], 0] == 255).all()
    # the Simple API on the same input gives the same colours
    s = R.image_synth(img, mask, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT))
    assert s.rc == 0 and (s.out[..., :nc] == r.out[..., 1:1 + nc]).all()


def test_batch_mixed_requests_and_errors(oracle):
    """One batch with random-order requests (shared launches), directional
    ones (host workers), replay-equivalent checks and per-request errors."""
    reqs = W.batch_requests(n=10, lo=40, hi=90, index=11)
    items = [(r["image"], r["mask"], r["fmt"], R.params(**r["params"])) for r in reqs]
    # requests 3 and 4 use the brushfire order (workers), 6 has an empty mask, 7 a mask of the wrong size
    items[3] = (items[3][0], items[3][1], items[3][2], R.params(**dict(reqs[3]["params"], matchContextType=2)))
    items[4] = (items[4][0], items[4][1], items[4][2], R.params(**dict(reqs[4]["params"], matchContextType=3)))
    items[6] = (items[6][0], np.zeros_like(items[6][1]), items[6][2], items[6][3])
    items[7] = (items[7][0], items[7][1][:-1], items[7][2], items[7][3])
    rc, outs, codes, st = R.image_synth_batch(items, opts=R.options(mode=R.MODE_WAVEFRONT), concurrency=3)
    assert codes[6] == 5      # IMAGE_SYNTH_ERROR_EMPTY_TARGET
    assert codes[7] == 2      # IMAGE_SYNTH_ERROR_IMAGE_MASK_MISMATCH
    assert rc == 5            # the first nonzero request result
    for i, (img, mask, fmt, p) in enumerate(items):
        if i in (6, 7):
            continue
        assert codes[i] == 0
        single = R.image_synth(img, mask, fmt, p, opts=R.options(mode=R.MODE_WAVEFRONT))
        assert single.rc == 0 and (single.out == outs[i]).all(), i
