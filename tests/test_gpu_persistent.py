"""The persistent wavefront pass (one cooperative launch per pass, a grid
barrier between batches) against one launch per batch, and its barrier's
bounded wait.  Integer work: outputs must be identical."""
import hashlib

import numpy as np
import pytest

import golden_cases as G
import resynthesizer_gb300 as R
from resynthesizer_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from resynthesizer_gb300 import build
    build.build()
    R.lib()


def _case(name):
    if name == "render":
        wl = W.render(tile=48, out=200)
        return wl["target"], wl["corpus"], wl["format"], wl["params"]
    if name == "render_tiled":
        wl = W.render(tile=40, out=120)
        return wl["target"], wl["corpus"], wl["format"], dict(wl["params"], tileH=1, tileV=1)
    if name == "heal":
        wl = W.heal4096(index=3, size=384)
        t, c = W.simple_to_pixmaps(wl["image"], wl["mask"])
        return t, c, (3, 0, 0, 0, 0), wl["params"]
    if name == "heal_brushfire":
        wl = W.heal_small(size=160, hole=90, ctype=2, patch=30, trys=100, index=4)
        t, c = W.simple_to_pixmaps(wl["image"], wl["mask"])
        return t, c, (3, 0, 0, 0, 0), wl["params"]
    wl = W.mapstyle(corpus_size=96, out=256, index=1)      # corpus read from global memory
    return wl["target"], wl["corpus"], wl["format"], wl["params"]


@pytest.mark.parametrize("name", ["render", "render_tiled", "heal", "heal_brushfire", "mapstyle"])
@pytest.mark.parametrize("warps", [0, 4])
def test_persistent_pass_equals_batch_launches(name, warps):
    t, c, spec, kw = _case(name)
    fmt = R.format_indices(*spec)
    a = R.engine(t, c, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT, warpsPerBlock=warps,
                                                           batchLaunches=2))
    b = R.engine(t, c, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT, warpsPerBlock=warps,
                                                           batchLaunches=1))
    assert a.rc == b.rc == 0, R.last_error()
    # (evals and terms may differ: a small batch's team of warps per target
    # depends on the grid size, and so does where each warp's early-outs fall)
    assert a.stats["passes"] == b.stats["passes"] and a.stats["betters"] == b.stats["betters"]
    assert np.array_equal(a.out, b.out)
    assert a.stats["launches"] < b.stats["launches"]


def test_persistent_launch_count_render1024():
    """render1024: the whole synthesis in a few dozen launches (one persistent
    launch per pass plus the per-pass bucketing), with the pinned output."""
    t, c, spec, kw = G.wave_workload("render1024")
    r = R.engine(t, c, R.format_indices(*spec), R.params(**kw),
                 opts=R.options(mode=R.MODE_WAVEFRONT, batchLaunches=2))
    assert r.rc == 0
    sha, npass, nbetter = G.WAVE_FULL["render1024"]
    assert hashlib.sha256(r.out.tobytes()).hexdigest() == sha
    assert r.stats["launches"] <= 50, r.stats["launches"]


def test_grid_barrier_passes_and_times_out():
    """Every CTA present: all barriers pass, no error.  One CTA absent: the
    others' waits give up after the time limit and report it, the kernel
    returns, and the context still runs a clean barrier test afterwards."""
    grid = 2 * R.sm_count()
    passed, err = R.grid_barrier_probe(5, -1, 2_000_000_000)
    assert (passed, err) == (5 * grid, 0)
    passed, err = R.grid_barrier_probe(5, 7, 20_000_000)          # 20 ms limit
    assert err & 4 and passed == 0
    passed, err = R.grid_barrier_probe(3, -1, 2_000_000_000)
    assert (passed, err) == (3 * grid, 0)


def test_persistent_cancel_mid_pass():
    """A cancel seen at a grid barrier stops every CTA at the same batch: the
    call returns 0 (the reference's rule) and the engine stays usable."""
    t, c, spec, kw = _case("heal")
    fmt = R.format_indices(*spec)
    r = R.engine(t, c, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT, batchLaunches=2), cancel=1)
    assert r.rc == 0
    again = R.engine(t, c, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT, batchLaunches=2))
    ref = R.engine(t, c, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT, batchLaunches=1))
    assert again.rc == 0 and np.array_equal(again.out, ref.out)


def test_launch_configuration_tuned_across_calls():
    """Without a fixed launch mode the first six calls of a problem class try,
    twice in turn, the persistent pass with 16 and 8 warps per CTA and one
    launch per batch; later calls use the fastest.  Every call gives the same
    output."""
    t, c, spec, kw = _case("render_tiled")
    kw = dict(kw, patchSize=12)                       # a class no other test uses
    fmt = R.format_indices(*spec)
    runs = [R.engine(t, c, fmt, R.params(**kw), opts=R.options(mode=R.MODE_WAVEFRONT)) for _ in range(8)]
    assert all(r.rc == 0 for r in runs)
    assert all(np.array_equal(r.out, runs[0].out) for r in runs[1:])
    modes = [r.stats["launchMode"] for r in runs]
    assert modes[:6] == [0, 1, 2, 0, 1, 2]            # persistent 16 and 8 warps, one launch per batch, twice
    assert modes[6] == modes[7] and modes[6] in (0, 1, 2)
    assert runs[0].stats["launches"] < runs[2].stats["launches"]
