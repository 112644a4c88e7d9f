"""The allocation-free frozen-state entry point (resynthFrozenBestFitNoAlloc).

It exists for callers that cannot let a library allocate device memory (a
host that hands out every GPU buffer from its own pool, or a latency-critical
loop that cannot take cudaMalloc's implicit synchronisation).  The test owns
every device buffer, calls the entry point through the C ABI twice in a row
with different problems -- so the second call runs over the working array the
first one left behind -- and requires results identical to the allocating
entry point resynthFrozenBestFit and to the CPU oracle's restatement of the
reference computeBestFit (integer metric: exact equality)."""
import ctypes as C

import numpy as np
import pytest

import resynthesizer_gb300 as R

pytestmark = pytest.mark.gpu


def _problem(seed, fmt, tw, th, cw, ch, tile, has_density=0.3, n=300):
    rng = np.random.default_rng(seed)
    bpp = 1 + fmt[0] + (1 if fmt[2] or fmt[3] else 0) + (fmt[1] if fmt[4] else 0)
    target = rng.integers(0, 256, (th, tw, bpp), dtype=np.uint8)
    corpus = rng.integers(0, 256, (ch, cw, bpp), dtype=np.uint8)
    corpus[..., 0] = np.where(rng.random((ch, cw)) < 0.9, 255, 0)
    has = (rng.random((th, tw)) < has_density).astype(np.uint8)
    src = np.full((th, tw, 2), -1, np.int32)
    m = rng.random((th, tw)) < 0.6
    src[m, 0] = rng.integers(0, cw, m.sum())
    src[m, 1] = rng.integers(0, ch, m.sum())
    targets = np.stack([rng.integers(0, tw, n), rng.integers(0, th, n)], 1).astype(np.int32)
    start = np.concatenate([[0], np.cumsum(rng.integers(0, 120, n))]).astype(np.uint32)
    cands = np.stack([rng.integers(-2, cw + 2, start[-1]), rng.integers(-2, ch + 2, start[-1])], 1).astype(np.int32)
    params = R.params(patchSize=int(rng.integers(5, 40)), mapWeight=0.6, tileH=tile, tileV=tile)
    return params, R.format_indices(*fmt), target, corpus, has, src, targets, start, cands


def _no_alloc(lib, params, fmt, target, corpus, has, src, targets, start, cands):
    import torch
    dev = torch.device("cuda", 0)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in dict(target=target, corpus=corpus, has=has, src=src, targets=targets,
                          start=start.view(np.int32), cands=cands).items()}
    n = len(targets)
    out_sum = torch.empty(n, dtype=torch.int32, device=dev)
    out_pt = torch.empty((n, 2), dtype=torch.int32, device=dev)
    out_cnt = torch.empty(n, dtype=torch.int32, device=dev)
    th, tw, _ = target.shape
    ch, cw, _ = corpus.shape
    stream = torch.cuda.current_stream(dev)
    vp = C.c_void_p
    rc = lib.resynthFrozenBestFitNoAlloc(
        C.byref(params), C.byref(fmt), vp(t["target"].data_ptr()), tw, th, vp(t["corpus"].data_ptr()), cw, ch,
        vp(t["has"].data_ptr()), vp(t["src"].data_ptr()), vp(t["targets"].data_ptr()), n,
        vp(t["start"].data_ptr()), vp(t["cands"].data_ptr()), vp(out_sum.data_ptr()), vp(out_pt.data_ptr()),
        vp(out_cnt.data_ptr()), vp(stream.cuda_stream))
    assert rc == 0, R.last_error()
    torch.cuda.synchronize(dev)
    return (out_sum.cpu().numpy().view(np.uint32), out_pt.cpu().numpy(), out_cnt.cpu().numpy().view(np.uint32))


@pytest.fixture(scope="module")
def lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from resynthesizer_gb300 import build
    build.build()
    L = R.lib()
    L.resynthFrozenBestFitNoAlloc.argtypes = [C.POINTER(R.ImageSynthParameters), C.POINTER(R.FormatIndices),
                                              C.c_void_p, C.c_uint, C.c_uint, C.c_void_p, C.c_uint, C.c_uint,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return L


def _oracle(oracle, params, fmt, *arrays):
    from oracle import Format, Params
    op = Params(params.isMakeSeamlesslyTileableHorizontally, params.isMakeSeamlesslyTileableVertically,
                params.matchContextType, params.mapWeight, params.sensitivityToOutliers, params.patchSize,
                params.maxProbeCount)
    of = Format(*(getattr(fmt, f) for f, _ in Format._fields_))
    return oracle.frozen(op, of, *arrays)


def _check(lib, oracle, prob):
    got = _no_alloc(lib, *prob)
    want = R.frozen_best_fit(*prob)
    ref = _oracle(oracle, *prob)
    for g, w, o in zip(got, want, ref):
        assert np.array_equal(g, w)
        assert np.array_equal(g, o)


def test_no_alloc_matches_allocating_entry_point_twice(lib, oracle):
    problems = [
        _problem(101, (3, 0, 0, 0, 0), 90, 70, 60, 50, 0),      # RGB, no maps
        _problem(202, (3, 1, 0, 0, 1), 64, 80, 100, 40, 1),     # RGB + one map channel, tiled
    ]
    for prob in problems:                                      # two calls in a row
        _check(lib, oracle, prob)


def test_no_alloc_thin_boxes_and_sparse_values(lib, oracle):
    # Thin and wide boxes with about 1 % of the pixels valued: patches are
    # gathered from far along the box; odd pixel counts leave the working
    # array's sections unaligned.
    problems = [
        _problem(303, (3, 0, 0, 0, 0), 3001, 3, 2001, 4, 0, has_density=0.01, n=200),
        _problem(404, (1, 0, 0, 0, 0), 2, 3999, 3, 1501, 0, has_density=0.01, n=200),
        _problem(505, (3, 1, 0, 0, 1), 4001, 2, 2999, 1, 1, has_density=0.02, n=150),
    ]
    for prob in problems:
        _check(lib, oracle, prob)


def test_no_alloc_rejects_oversized_images(lib):
    p = R.params()
    f = R.format_indices(3)
    big = 2048
    rc = lib.resynthFrozenBestFitNoAlloc(C.byref(p), C.byref(f), C.c_void_p(1), big, big, C.c_void_p(1), big, big,
                                         C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), 0, C.c_void_p(1),
                                         C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), None)
    assert rc == 101 and "8 MiB" in R.last_error()


def test_no_alloc_call_captured_in_graph(lib):
    # After the first call on a device, a call enqueues kernels only (the
    # metric tables travel as kernel arguments), so it can be captured into a
    # CUDA graph.  Another problem with other metric parameters runs between
    # capture and replay: the replay rewrites the whole working array itself.
    import torch
    dev = torch.device("cuda", 0)
    prob = _problem(606, (3, 1, 0, 0, 1), 70, 60, 80, 50, 0)
    params, fmt, target, corpus, has, src, targets, start, cands = prob
    params.sensitivityToOutliers = 0.3
    want = _no_alloc(lib, *prob)
    other = _problem(707, (3, 0, 0, 0, 0), 50, 40, 60, 30, 1)
    other[0].sensitivityToOutliers = 0.05
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev)
         for k, v in dict(target=target, corpus=corpus, has=has, src=src, targets=targets,
                          start=start.view(np.int32), cands=cands).items()}
    n = len(targets)
    outs = [torch.zeros(n, dtype=torch.int32, device=dev), torch.zeros((n, 2), dtype=torch.int32, device=dev),
            torch.zeros(n, dtype=torch.int32, device=dev)]
    th, tw, _ = target.shape
    ch, cw, _ = corpus.shape
    vp = C.c_void_p
    torch.cuda.synchronize(dev)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        rc = lib.resynthFrozenBestFitNoAlloc(
            C.byref(params), C.byref(fmt), vp(t["target"].data_ptr()), tw, th, vp(t["corpus"].data_ptr()), cw, ch,
            vp(t["has"].data_ptr()), vp(t["src"].data_ptr()), vp(t["targets"].data_ptr()), n,
            vp(t["start"].data_ptr()), vp(t["cands"].data_ptr()), vp(outs[0].data_ptr()), vp(outs[1].data_ptr()),
            vp(outs[2].data_ptr()), vp(torch.cuda.current_stream(dev).cuda_stream))
    assert rc == 0, R.last_error()
    _no_alloc(lib, *other)
    g.replay()
    torch.cuda.synchronize(dev)
    got = (outs[0].cpu().numpy().view(np.uint32), outs[1].cpu().numpy(), outs[2].cpu().numpy().view(np.uint32))
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
