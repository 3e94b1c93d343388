"""Learned warm start: the library's forward/backward kernels against the
float64 numpy restatement (oracle/warmstart_ref.py), then a small
experiment at 128x128: the potential-well state plus the correction
trained on solver equilibria must reach the same equilibrium as the
Gaussian start in fewer periods.  Both runs stop when the profile changes
by less than 1e-5 per period, which leaves each within about a damping
time of that change (~1e-3) of the fixed point: the two end states must
agree to relative L1 <= 3e-3.

Gradient tolerance: each gradient within 2e-3 of its largest entry (BF16
weights are used exactly on both sides; the GPU sums in FP32)."""
import numpy as np
import pytest

from oracle import warmstart_ref as R
from inovesa_gb300 import warmstart as W

pytestmark = pytest.mark.gpu


def test_ws_gradients_match_reference(gpu_ctx):
    npix, B = 4096, 8
    net = W.WarmStartNet(gpu_ctx, npix, seed=3)
    rng = np.random.default_rng(4)
    net.set_bias(rng.normal(0, 0.1, size=npix))
    x = rng.normal(size=(B, 3)).astype(np.float32)
    t = rng.normal(0, 0.1, size=(B, npix)).astype(np.float32)
    # a few updates so that every layer has non-trivial weights
    for _ in range(3):
        net.train_step(x, t, lr=1e-2)
    loss, g = net.gradients(x, t)
    w = net.weights_bf16()
    rloss, rg = R.loss_and_grads(w, x, t)
    assert abs(loss - rloss) <= 1e-5 * rloss
    for k in rg:
        m = np.abs(rg[k]).max()
        assert np.abs(g[k] - rg[k]).max() <= 2e-3 * m, k
    y = net.forward(x)
    assert np.abs(y - R.forward(w, x)[3]).max() <= 1e-4


def test_ws_small_experiment(gpu_ctx):
    res, _ = W.experiment(gpu_ctx, n=128, spt=500, ntrain=192, ntest=24,
                          iters=1500, max_periods=200, seed=11)
    print(res)
    assert res["train_loss_last"] < 0.5 * res["train_loss_first"]
    assert res["test_converged_all"] >= 0.8 * res["test_converged_gaussian"]
    assert res["same_equilibrium_l1_max"] <= 3e-3
    assert res["proposal_l1_median"] <= 5e-3
    assert res["speedup_median"] >= 1.5
    assert res["periods_warm_median"] < res["periods_gaussian_median"]
