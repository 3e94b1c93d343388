"""Learned warm start: the library's forward/backward kernels against the
float64 numpy restatement (oracle/warmstart_ref.py), then the experiment
on 256x256 bunches (the benchmark's mesh): the potential-well state plus
the correction trained on solver equilibria, on held-out inputs (S, g/R,
damping time from 5 to 150 synchrotron periods), must

* reach equilibrium at least 5x faster than the Gaussian start (median
  over the bunches of the ratio of periods),
* reach it faster than the potential-well state alone (what the trained
  network itself adds: median periods lower, and more bunches faster than
  slower),
* reach the same equilibrium as the Gaussian start (the solver is the
  judge): both runs stop once the profile has changed by less than 1e-5
  per period for three periods in a row, which leaves each a few damping
  times' worth of that change from the fixed point (up to ~1e-3 at 150
  periods); the end states must agree to relative L1 <= 1e-3 in the median
  and <= 1e-2 for every bunch (the Gaussian start of a long-damped bunch
  can stop while a slow coherent mode still rings).

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


def test_ws_experiment_256(gpu_ctx):
    res, _ = W.experiment(gpu_ctx, n=256, spt=1000, ntrain=512, ntest=24,
                          iters=2000, max_periods=600, seed=11)
    print(res)
    assert res["train_loss_last"] < 0.5 * res["train_loss_first"]
    # a long-damped bunch's Gaussian start may not settle within the 600
    # periods; such bunches stay out of the ratios
    assert res["test_converged_all"] >= 0.75 * res["test_samples"]
    assert res["same_equilibrium_l1_median"] <= 1e-3
    assert res["same_equilibrium_l1_max"] <= 1e-2
    assert res["speedup_median"] >= 5.0
    assert (res["periods_warm_median"]
            < res["periods_potential_well_median"])
    assert (res["warm_faster_than_potential_well"]
            > res["warm_slower_than_potential_well"])
