"""The CPU oracle against the golden fixtures made by the reference engine
(tests/golden/make_golden.py).  Needs no reference tree, so it also pins the
oracle on machines that only have the committed fixtures."""
import hashlib

import numpy as np
import pytest

import golden_cases as G
from oracle import make_params


def test_testsynth_known_answers(oracle):
    for case in G.testsynth():
        p = make_params(**case["params"]) if case["params"] else None
        rc, out, _ = oracle.image_synth(case["image"], case["mask"], case["fmt"], p)
        assert rc == case["rc"], case["name"]
        assert (out == case["out"]).all(), case["name"]


@pytest.mark.parametrize("k", range(16))
def test_heal_cases(oracle, k):
    case = G.heal()[k]
    rc, out, _ = oracle.image_synth(case["image"], case["mask"], case["fmt"], make_params(**case["params"]))
    assert rc == 0 and (out == case["out"]).all()


def test_heal256(oracle):
    case = G.heal256()
    rc, out, st = oracle.image_synth(case["image"], case["mask"], case["fmt"], make_params(**case["params"]))
    assert rc == 0
    assert (out[96:160, 96:160] == case["out_region"]).all()
    assert hashlib.sha256(out.tobytes()).hexdigest() == case["sha256"]


def test_engine_cases(oracle):
    for case in G.engine():
        fmt = oracle.format_indices(*case["format"])
        rc, t, _, s, h = oracle.engine(make_params(**case["params"]), fmt, case["target"], case["corpus"],
                                       want_state=True)
        assert rc == 0, case["name"]
        assert (t == case["out"]).all() and (s == case["source"]).all() and (h == case["has"]).all(), case["name"]


def test_frozen_cases(oracle):
    for case in G.frozen():
        fmt = oracle.format_indices(*case["format"])
        s, pt, cnt = oracle.frozen(make_params(**case["params"]), fmt, case["target"], case["corpus"], case["has"],
                                   case["source"], case["targets"], case["start"], case["cands"])
        assert (s == case["sum"]).all() and (pt == case["pt"]).all() and (cnt == case["count"]).all()
