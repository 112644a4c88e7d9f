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
