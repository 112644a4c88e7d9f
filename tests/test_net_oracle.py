"""The proposal network's CPU oracle checked against itself: analytic
gradients against central finite differences (rounding off, float64), the
im2col/col2im adjoint identity and the loss's winner weighting."""
import numpy as np

import proposal_net as N


def _case(n=3, seed=1):
    rng = np.random.default_rng(seed)
    theta = N.init_params(seed).astype(np.float64)
    x0 = rng.uniform(-0.5, 0.5, (n, N.CTX, N.CTX, N.CIN0))
    x0[..., 5:] = 0.0
    labels = rng.uniform(-3, 3, (n, 2))
    return theta, x0, labels


def test_param_count():
    assert N.param_count() == 32 * 144 + 32 + 4 * (32 * 288 + 32)


def test_im2col_col2im_adjoint():
    rng = np.random.default_rng(0)
    a = rng.standard_normal((2, 7, 7, 4))
    d = rng.standard_normal((2 * 25, 36))
    assert np.isclose((N.im2col(a) * d).sum(), (a * N.col2im(d, 2, 7, 4)).sum())


def test_gradient_matches_finite_differences():
    theta, x0, labels = _case()
    _, g = N.loss_and_grad(theta, x0, labels, rounding=False)
    rng = np.random.default_rng(5)
    idx = rng.choice(theta.size, 60, replace=False)
    # include every layer's biases and the head
    idx = np.concatenate([idx, [32 * 144 + 3, N.param_count() - 1, N.param_count() - 40]])
    h = 1e-6
    for i in idx:
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        lp = N.mcl_loss(N.forward(tp, x0, rounding=False)[0], labels)[0]
        lm = N.mcl_loss(N.forward(tm, x0, rounding=False)[0], labels)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])


def test_loss_weights_nearest_offset():
    out = np.zeros((1, 32))
    out[0, 2:4] = [1.0, 1.0]          # offset 1 sits on the label
    loss, grad = N.mcl_loss(out, np.array([[1.0, 1.0]]))
    # winner contributes 0; the 15 others each |0 - (1,1)|^2 = 2 with weight EPS/15
    assert np.isclose(loss, N.EPS / 15 * 2 * 15)
    assert np.allclose(grad[0, 2:4], 0.0)
