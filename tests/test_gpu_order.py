"""The directional and brushfire visit orders (matchContextType 2..8) made on
the device against the oracle's restatement, which sorts with libc qsort and
the reference's comparators (lib/orderTarget.h:268-343, lib/brushfire.h:62-163)
and draws the banded shuffle from libc rand: exact equality of the order."""
import numpy as np
import pytest

import resynthesizer_gb300 as R

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from resynthesizer_gb300 import build
    build.build()
    R.lib()


def _row_major(mask):
    ys, xs = np.nonzero(mask)
    return np.stack([xs, ys], 1).astype(np.int32)


def _shapes():
    rng = np.random.default_rng(5)
    out = {}
    m = np.zeros((64, 64), bool)
    m[16:48, 20:44] = True                             # a square hole: ties on axes and diagonals
    out["square"] = m
    m = np.zeros((90, 70), bool)
    yy, xx = np.mgrid[0:90, 0:70]
    m[(yy - 45) ** 2 / 900 + (xx - 33) ** 2 / 400 < 1] = True
    out["ellipse"] = m
    out["sparse"] = rng.random((120, 100)) < 0.05
    m = np.zeros((41, 41), bool)
    m[20, 20] = True                                   # the centre alone on its ray: a NaN key
    m[5, 5] = m[35, 8] = m[3, 30] = True
    out["centre_alone"] = m
    m = np.zeros((30, 200), bool)
    m[10:20, 3:197] = True                             # wide band, ties of |dy|
    out["wide"] = m
    m = np.zeros((1, 50), bool)
    m[0, 10:40] = True                                 # one row
    out["row"] = m
    m = np.zeros((300, 300), bool)
    m[40:260, 40:260] = rng.random((220, 220)) < 0.7   # many targets: several sort chunks
    out["large"] = m
    return out


SHAPES = _shapes()


@pytest.mark.parametrize("name", sorted(SHAPES))
@pytest.mark.parametrize("ctype", range(2, 9))
def test_device_order_equals_reference_order(oracle, name, ctype):
    pts = _row_major(SHAPES[name])
    want = oracle.order_targets(ctype, pts)
    got = R.order_targets_device(ctype, pts)
    assert np.array_equal(got, want)
