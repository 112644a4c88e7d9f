"""The learned-proposal network's tensor-core kernels against fp32 references
computed on the CPU from the same bf16-rounded operands."""
import numpy as np
import pytest

import resynthesizer_gb300 as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from resynthesizer_gb300 import build
    build.build()
    R.lib()


def bf16(x):
    """Round float32 to the nearest even bfloat16, returned as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


def test_bounded_wait_reports_and_context_survives():
    # a barrier that never completes: the kernel gives up, flags the error and
    # frees its tensor memory; the next GEMM on the same context is correct
    rc = R.lib().resynthTcWaitTimeout()
    assert rc == 100 and "ran out" in R.last_error()
    a = np.random.default_rng(1).standard_normal((128, 32)).astype(np.float32)
    d = R.tc_gemm(a, a)
    ref = bf16(a).astype(np.float64) @ bf16(a).astype(np.float64).T
    np.testing.assert_allclose(d, ref, rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("m,n,k", [(128, 32, 16), (128, 32, 64), (300, 96, 288), (1000, 32, 80),
                                   (257, 64, 600)])
def test_tc_gemm_matches_fp32(m, n, k):
    rng = np.random.default_rng(m * 7 + n + k)
    a = rng.standard_normal((m, k)).astype(np.float32)
    b = rng.standard_normal((n, k)).astype(np.float32)
    d = R.tc_gemm(a, b)
    ref = bf16(a).astype(np.float64) @ bf16(b).astype(np.float64).T
    # fp32 accumulation of k products of bf16 values: relative error ~ k * 2^-24
    np.testing.assert_allclose(d, ref, rtol=1e-4, atol=1e-4 * np.sqrt(k))


# ------------------------------------------------------------ the network

import proposal_net as N   # noqa: E402


def _contexts(n, seed):
    """Contexts with the engine's channel structure: colours where valued, a
    has-value channel, a map channel, zeros elsewhere."""
    rng = np.random.default_rng(seed)
    x = np.zeros((n, 11, 11, 16), np.float32)
    has = rng.random((n, 11, 11)) < 0.6
    x[..., 0:3] = (rng.integers(0, 256, (n, 11, 11, 3)) / np.float32(255) - 0.5) * has[..., None]
    x[..., 3] = has
    x[..., 4] = rng.integers(0, 256, (n, 11, 11)) / np.float32(255) - 0.5
    return N.bf16_bits(x)


@pytest.fixture(scope="module")
def net():
    n = R.Net(seed=3)
    yield n
    n.close()


@pytest.mark.parametrize("n", [1, 37, 300])
@pytest.mark.parametrize("path", [0, 1])
def test_net_forward_matches_oracle(net, n, path):
    theta = net.get_params()
    x = _contexts(n, seed=n)
    out = net.forward(x, path=path)
    ref, _ = N.forward(theta, N.bits_to_float(x))
    # bf16 activations: a rounding flip between fp32 (GPU) and float64 sums
    # moves an output by ~2^-8 of its scale
    scale = np.abs(ref).max()
    np.testing.assert_allclose(out, ref, rtol=2e-2, atol=2e-2 * scale)
    assert np.abs(out - ref).mean() < 2e-3 * scale


def test_net_paths_agree(net):
    x = _contexts(200, seed=9)
    a, b = net.forward(x, path=0), net.forward(x, path=1)
    np.testing.assert_allclose(a, b, rtol=1e-2, atol=1e-2 * np.abs(b).max())


@pytest.mark.parametrize("n", [5, 64])
def test_net_gradients_match_oracle(net, n):
    theta = net.get_params()
    x = _contexts(n, seed=100 + n)
    labels = np.random.default_rng(n).uniform(-2, 2, (n, 2)).astype(np.float32)
    loss, g = net.gradients(x, labels)
    ref_loss, ref_g = N.loss_and_grad(theta, N.bits_to_float(x), labels)
    assert abs(loss - ref_loss) <= 1e-3 * abs(ref_loss) + 1e-6
    o = 0
    for cin, _ in N.LAYERS:
        for size in (32 * 9 * cin, 32):
            a, b = g[o:o + size], ref_g[o:o + size]
            o += size
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            assert rel < 2e-2, (o, rel)


def test_net_training_reduces_loss():
    # labels that are a function of the context: the mean of colour 0 over
    # the valued pixels and the valued fraction
    n = 4096
    x = _contexts(n, seed=7)
    xf = N.bits_to_float(x)
    has = xf[..., 3]
    lab = np.stack([4 * (xf[..., 0] * has).sum((1, 2)) / np.maximum(has.sum((1, 2)), 1),
                    4 * has.mean((1, 2)) - 2], -1).astype(np.float32)
    net = R.Net(seed=11)
    pairs = R.Pairs(n)
    assert pairs.add(x, lab) == n and len(pairs) == n
    rx, ry = pairs.read(10, 5)
    assert np.array_equal(rx, x[10:15]) and np.array_equal(ry, lab[10:15])
    before, _ = net.gradients(x[:512], lab[:512])
    after = net.train(pairs, steps=300, batch=256, lr=2e-3)
    final, _ = net.gradients(x[:512], lab[:512])
    assert final < 0.3 * before, (before, after, final)
    net.close()
    pairs.close()


def test_net_training_is_deterministic():
    # the weight and bias gradients are summed in a fixed order (no float
    # atomics): two networks trained alike end with identical parameters
    n = 2048
    x = _contexts(n, seed=9)
    lab = np.random.default_rng(9).standard_normal((n, 2)).astype(np.float32)
    pairs = R.Pairs(n)
    assert pairs.add(x, lab) == n
    a, b = R.Net(seed=13), R.Net(seed=13)
    a.train(pairs, steps=40, batch=512, lr=1e-3)
    b.train(pairs, steps=40, batch=512, lr=1e-3)
    assert np.array_equal(a.get_params(), b.get_params())
    for o in (a, b, pairs):
        o.close()


# ------------------------------------------------- the network in synthesis

from resynthesizer_gb300 import workloads as W   # noqa: E402


def test_dump_pairs_match_final_state():
    wl = W.render(tile=48, out=64)
    tgt, cor, kw = wl["target"], wl["corpus"], wl["params"]
    fmt = R.format_indices(*wl["format"])
    pairs = R.Pairs(100000)
    stride = 7
    r = R.engine(tgt, cor, fmt, R.params(**kw),
                 opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1, dump=pairs, dumpStride=stride))
    assert r.rc == 0
    ys, xs = np.nonzero(tgt[..., 0] != 0)          # targets in raster order
    pos = np.stack([xs, ys], 1)[::stride]
    assert len(pairs) == len(pos)
    x, lab = pairs.read()
    colors = r.out[..., 1:1 + fmt.img_match_bpp]
    valued = r.has_value.astype(bool)
    src = r.source
    for i in range(len(pos)):
        tx, ty = pos[i]
        assert lab[i, 0] == np.float32(src[ty, tx, 0] - tx) / 64 and lab[i, 1] == np.float32(src[ty, tx, 1] - ty) / 64
        if i % 2:
            # complete context: exactly the final image around the target
            assert np.array_equal(x[i], N.context(colors, valued, None, tx, ty)), i
        else:
            # the context at the target's first visit: a subset of the final
            # one with the same colours where it has values
            full = N.bits_to_float(N.context(colors, valued, None, tx, ty))
            part = N.bits_to_float(x[i])
            h = part[..., 3] > 0
            assert (full[..., 3][h] > 0).all() and np.array_equal(part[h], full[h])
            assert not h[5, 5]             # the target itself had no value yet
    pairs.close()


def test_map_guided_proposals():
    """Map-conditioned proposals (the survey's map-guided style transfer): the
    dumped contexts carry the target map's first channel where the reference
    would see it, a network trained on them proposes sources for a map-guided
    synthesis, and that synthesis keeps every invariant and is deterministic."""
    wl = W.mapstyle(corpus_size=48, out=96, index=3)
    tgt, cor, kw = wl["target"], wl["corpus"], wl["params"]
    fmt = R.format_indices(*wl["format"])
    pairs = R.Pairs(100000)
    r = R.engine(tgt, cor, fmt, R.params(**kw),
                 opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1, dump=pairs, dumpStride=5))
    assert r.rc == 0
    ys, xs = np.nonzero(tgt[..., 0] != 0)
    pos = np.stack([xs, ys], 1)[::5]
    x, lab = pairs.read()
    assert len(x) == len(pos)
    mapc = tgt[..., fmt.map_start_bip]
    colors = r.out[..., 1:1 + fmt.img_match_bpp]
    for i in range(1, len(pos), 2):                # complete contexts: the final image and the map
        tx, ty = pos[i]
        assert np.array_equal(x[i], N.context(colors, r.has_value.astype(bool), mapc, tx, ty)), i
    net = R.Net(seed=4)
    net.train(pairs, steps=300, batch=256, lr=1e-3)
    runs = [R.engine(tgt, cor, fmt, R.params(**kw),
                     opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1, net=net, proposals=16)) for _ in range(2)]
    assert all(q.rc == 0 for q in runs) and np.array_equal(runs[0].out, runs[1].out)
    q = runs[0]
    sel = tgt[..., 0] != 0
    src = q.source[sel]
    assert (src[:, 0] >= 0).all()
    assert (q.out[sel][:, 1:4] == cor[src[:, 1], src[:, 0], 1:4]).all()
    assert (q.out[..., fmt.map_start_bip] == tgt[..., fmt.map_start_bip]).all()
    net.close()
    pairs.close()


def _heal_run(wl, net=None, proposals=0, trys=None):
    tgt, cor = W.simple_to_pixmaps(wl["image"], wl["mask"])
    kw = dict(wl["params"])
    if trys is not None:
        kw["maxProbeCount"] = trys
    fmt = R.format_indices(3, 0, 0, 0, 0)
    r = R.engine(tgt, cor, fmt, R.params(**kw),
                 opts=R.options(mode=R.MODE_WAVEFRONT, recordState=1, net=net, proposals=proposals))
    assert r.rc == 0
    sel = tgt[..., 0] != 0
    ys, xs = np.nonzero(sel)
    targets = np.stack([xs, ys], 1).astype(np.int32)
    e, _ = R.patch_energy(R.params(**kw), fmt, r.out, cor, r.has_value, r.source, targets)
    return r, e, tgt, cor, sel


def test_wavefront_with_proposals_keeps_invariants(net):
    wl = W.heal_small(size=96, hole=40, ctype=2, patch=30, trys=200)
    r, e, tgt, cor, sel = _heal_run(wl, net=net, proposals=16)
    r2, e2, *_ = _heal_run(wl, net=net, proposals=16)
    assert (r.out == r2.out).all() and e == e2          # deterministic
    assert (r.out[~sel] == tgt[~sel]).all()
    src = r.source[sel]
    assert (src[:, 0] >= 0).all() and r.has_value[sel].all()
    assert (r.out[sel][:, 1:4] == cor[src[:, 1], src[:, 0], 1:4]).all()
    assert r.stats["evals"] > 0
    # only the network's candidates and the continuations: still a valid synthesis
    r0, e0, *_ = _heal_run(wl, net=net, proposals=16, trys=0)
    assert (r0.source[sel][:, 0] >= 0).all()


def test_trained_network_gain():
    """What the trained network gains over the search without it, at equal
    probe counts (16 proposals + 16 random probes against 16 random probes),
    on a held-out 256x256 heal of seeded value noise.

    * Trained on the pairs of a plain run of the same image (contexts as at
      each target's first visit, labels the final sources): it lowers the
      patch energy (by about 8 % here), and beats the untrained network.
    * Trained on pairs from four other images: value noise shares no structure
      across images, and the network gains nothing reliable over the random
      probes -- it is asserted to do no better than the same-image network.
    * With no random probes at all the continuations alone cannot start a
      heal (no context pixel has a source): any network's proposals are then
      the only new candidates, and the trained one beats the untrained one.
    The training also lowers the loss on pairs from the held-out run."""
    fmt = R.format_indices(3, 0, 0, 0, 0)

    def dump(wl, pairs):
        tgt, cor = W.simple_to_pixmaps(wl["image"], wl["mask"])
        r = R.engine(tgt, cor, fmt, R.params(**wl["params"]),
                     opts=R.options(mode=R.MODE_WAVEFRONT, dump=pairs, dumpStride=1))
        assert r.rc == 0

    wl0 = W.heal4096(index=0, size=256)
    other, same = R.Pairs(400000), R.Pairs(100000)
    for i in range(2, 6):
        dump(W.heal4096(index=i, size=256), other)
    dump(wl0, same)
    hx, hy = same.read()
    untrained, cross, self_ = R.Net(seed=21), R.Net(seed=21), R.Net(seed=21)
    cross.train(other, steps=600, batch=512, lr=1e-3)
    self_.train(same, steps=600, batch=512, lr=1e-3)
    assert self_.gradients(hx, hy)[0] < untrained.gradients(hx, hy)[0]
    assert cross.gradients(hx, hy)[0] < untrained.gradients(hx, hy)[0]
    _, e_plain, *_ = _heal_run(wl0, trys=16)
    _, e_self, *_ = _heal_run(wl0, net=self_, proposals=16, trys=16)
    _, e_untrained, *_ = _heal_run(wl0, net=untrained, proposals=16, trys=16)
    _, e_cross, *_ = _heal_run(wl0, net=cross, proposals=16, trys=16)
    assert e_self < 0.97 * e_plain, (e_self, e_plain)
    assert e_self < e_untrained, (e_self, e_untrained)
    assert e_cross > e_self, (e_cross, e_self)
    _, p0, *_ = _heal_run(wl0, trys=0)
    _, u0, *_ = _heal_run(wl0, net=untrained, proposals=16, trys=0)
    _, t0, *_ = _heal_run(wl0, net=self_, proposals=16, trys=0)
    assert t0 < u0 < 0.5 * p0, (t0, u0, p0)
    for o in (other, same, untrained, cross, self_):
        o.close()
