"""The wavefront oracle (oracle/wave_oracle.c): a plain-C restatement of the
library's default mode -- random visit order by a pixel hash, bands of
f, 2f, 4f ... targets (f = 16, or n / 1024 for heals) cut into k x k colour
phases, visit stamps, patches
from the sorted offsets within min(box diagonal, 256), deduplicated
continuations then counter-hashed probes, the first strict minimum of the
patch metric, staged stores, the reference's stop rule.  Its outputs on the
full-size workloads are pinned by hash (the CUDA library's outputs on a
GB300 hash the same: tests/test_gpu_parity.py), and on small cases it is
checked against the invariants every engine output has."""
import hashlib

import numpy as np
import pytest

import golden_cases as G
from oracle import Oracle, make_params
from resynthesizer_gb300 import workloads as W


@pytest.fixture(scope="module")
def oracle():
    return Oracle()


@pytest.mark.parametrize("name", ["render1024", "heal4096"])
def test_wave_oracle_full_size_pinned(oracle, name):
    t, c, spec, kw = G.wave_workload(name)
    rc, out, passes, betters = oracle.wave_engine(make_params(**kw), oracle.format_indices(*spec), t, c, threads=8)
    sha, npass, nbetter = G.WAVE_FULL[name]
    assert rc == 0
    assert (passes, betters) == (npass, nbetter)
    assert hashlib.sha256(out.tobytes()).hexdigest() == sha


@pytest.mark.parametrize("case", sorted(G.WAVE_SMALL))
def test_wave_oracle_small_cases_pinned(oracle, case):
    t, c, spec, kw = G.wave_small_case(case)
    rc, out, passes, betters = oracle.wave_engine(make_params(**kw), oracle.format_indices(*spec), t, c)
    sha, npass, nbetter = G.WAVE_SMALL[case]
    assert rc == 0 and (passes, betters) == (npass, nbetter)
    assert hashlib.sha256(out.tobytes()).hexdigest() == sha


@pytest.mark.parametrize("threads", [1, 3])
def test_wave_oracle_threads_and_invariants(oracle, threads):
    """Same output for any thread count; only target colours change, and every
    target pixel ends with the colours of some corpus pixel."""
    wl = W.heal_small(size=40, hole=12, ctype=1, patch=16, trys=60)
    t, c = W.simple_to_pixmaps(wl["image"], wl["mask"])
    p, fmt = make_params(**wl["params"]), oracle.format_indices(3, 0, 0, 0, 0)
    rc, out, passes, betters = oracle.wave_engine(p, fmt, t, c, threads=threads)
    rc8, out8, _, _ = oracle.wave_engine(p, fmt, t, c, threads=8)
    assert rc == rc8 == 0 and np.array_equal(out, out8)
    sel = t[..., 0] != 0
    assert np.array_equal(out[~sel], t[~sel]) and np.array_equal(out[..., 0], t[..., 0])
    corpus_cols = {tuple(v) for v in c[c[..., 0] == 0xFF][:, 1:4]}
    assert all(tuple(v) in corpus_cols for v in out[sel][:, 1:4])
    assert 1 <= passes <= 6 and betters[0] == int(sel.sum())


@pytest.mark.parametrize("ctype", [2, 5, 8])
def test_wave_oracle_directional_orders(oracle, ctype):
    """Directional orders (the reference's own visit order, bands of equal
    width): deterministic, and the same invariants."""
    wl = W.heal_small(size=40, hole=12, ctype=ctype, patch=16, trys=40, index=ctype)
    t, c = W.simple_to_pixmaps(wl["image"], wl["mask"])
    p, fmt = make_params(**wl["params"]), oracle.format_indices(3, 0, 0, 0, 0)
    rc, out, passes, betters = oracle.wave_engine(p, fmt, t, c, threads=1)
    rc2, out2, _, _ = oracle.wave_engine(p, fmt, t, c, threads=4)
    assert rc == rc2 == 0 and np.array_equal(out, out2)
    sel = t[..., 0] != 0
    assert np.array_equal(out[~sel], t[~sel]) and betters[0] == int(sel.sum())


def test_wave_oracle_rejects_unknown_order(oracle):
    wl = W.heal_small(size=24, hole=8, ctype=1, patch=9, trys=20)
    t, c = W.simple_to_pixmaps(wl["image"], wl["mask"])
    rc, _, _, _ = oracle.wave_engine(make_params(**dict(wl["params"], matchContextType=9)),
                                     oracle.format_indices(3, 0, 0, 0, 0), t, c)
    assert rc == -1
