"""Particle tracking through the Fokker-Planck map
(FokkerPlanckMap::applyTo, src/SM/FokkerPlanckMap.cpp:214-268), through the
C ABI (vfps_map_apply_to), against the oracle's restatement
(oracle.fp_particle).

* approximation1 and approximation2 are deterministic float arithmetic on
  the map's stencil table (and, for approximation2, the input density):
  compared with the restatement at 1 ulp-level tolerance (2e-6 of the
  position), for both derivations and all FP types.
* stochastic draws from N(0, sqrt(2 e1)/dp) (the reference seeds its
  generator from std::random_device, so only the distribution can agree):
  the mean displacement -y e1 and the spread sqrt(2 e1)/dp are checked on
  2e5 draws within 5 standard errors, and no draw is repeated between two
  calls.
"""
import math

import numpy as np
import pytest

import oracle
from inovesa_gb300 import vfps as V

pytestmark = pytest.mark.gpu

AXES = (-6.0, 6.0, 2e-3, -6.0, 6.0, 6.11e5)


def density(n, seed=0):
    rng = np.random.default_rng(seed)
    q = np.linspace(-6, 6, n)
    g = np.exp(-0.5 * (q[:, None] ** 2 + (q[None, :] - 0.4) ** 2))
    g *= 1 + 0.2 * np.sin(q[:, None] + 0.7 * q[None, :])
    g += 1e-3 * rng.random((n, n))
    return (g / g.sum()).astype(np.float32)[None]


def particles(n, count, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(1.0, n - 1.0, size=(count, 2)).astype(np.float32)
    # a few on cell boundaries, next to both edges and around the centre
    pos[:6, 1] = [1.0, 2.0, n / 2 - 1, n / 2, n - 2.0, n - 1.5]
    return pos


@pytest.mark.parametrize("derivation", [3, 4])
@pytest.mark.parametrize("fptype", [1, 2, 3])
@pytest.mark.parametrize("mode", [1, 2])
def test_fp_tracking_deterministic(gpu_ctx, derivation, fptype, mode):
    n = 128
    e1 = 2.0 / (100 * 500) * 50
    d = density(n, seed=derivation + 10 * fptype)
    a = V.PhaseSpace(*AXES, gpu_ctx, 1, 1, [1.0], 1.0, d, n=n)
    b = V.PhaseSpace(*AXES, gpu_ctx, 1, 1, [1.0], 1.0, None, n=n)
    m = V.FokkerPlanckMap(a, b, n, n, fptype, mode, e1, derivation)
    pos = particles(n, 300, seed=mode + derivation + fptype)
    got = m.applyTo(pos.copy())
    idx, w = oracle.fp_stencils(n, AXES, e1, fptype, derivation,
                                dtype=np.float32)
    want = oracle.fp_particle(mode, n, derivation, idx, w, pos,
                              density=a.getData())
    np.testing.assert_array_equal(np.asarray(got)[:, 0], pos[:, 0])
    np.testing.assert_allclose(np.asarray(got)[:, 1], want[:, 1], rtol=0,
                               atol=2e-6 * n)
    # the map moves particles (a table of zeros would pass the above only
    # with an all-zero restatement too); the diffusion-only stencil is
    # symmetric, so its mean displacement (approximation1) is zero
    if not (mode == 1 and fptype == 2):
        assert np.abs(want[:, 1] - pos[:, 1]).max() > 1e-4


def test_fp_tracking_stochastic(gpu_ctx):
    n = 128
    e1 = 2.0 / (100 * 500)
    a = V.PhaseSpace(*AXES, gpu_ctx, 1, 1, [1.0], 1.0, density(n), n=n)
    b = V.PhaseSpace(*AXES, gpu_ctx, 1, 1, [1.0], 1.0, None, n=n)
    m = V.FokkerPlanckMap(a, b, n, n, 3, 3, e1, 4)
    count = 200_000
    y0 = np.float32(70.25)
    pos = np.zeros((count, 2), np.float32)
    pos[:, 0] = 10.0
    pos[:, 1] = y0
    got1 = np.asarray(m.applyTo(pos.copy()))
    got2 = np.asarray(m.applyTo(pos.copy()))
    dp = (AXES[4] - AXES[3]) / (n - 1)
    sigma = math.sqrt(2 * e1) / dp
    for got in (got1, got2):
        np.testing.assert_array_equal(got[:, 0], pos[:, 0])
        shift = y0 - got[:, 1].astype(np.float64)   # = y e1 + noise
        mean_want = float(y0) * e1
        se = sigma / math.sqrt(count)
        assert abs(shift.mean() - mean_want) < 5 * se, (shift.mean(),
                                                        mean_want, se)
        sd = shift.std()
        assert abs(sd - sigma) < 5 * sigma / math.sqrt(2 * count), (sd,
                                                                    sigma)
        # Gaussian shape: the fourth standardised moment is 3
        z = (shift - shift.mean()) / sd
        assert abs((z ** 4).mean() - 3.0) < 0.1
    # independent draws between calls
    assert np.mean(got1[:, 1] == got2[:, 1]) < 0.01
    # the restatement with the same noise reproduces the call exactly
    noise = (y0 - got1[:, 1].astype(np.float64)) - float(y0) * e1
    want = oracle.fp_particle(3, n, 4, np.zeros(4 * n), np.zeros(4 * n),
                              pos[:50], e1=e1, dp=dp, noise=noise[:50])
    np.testing.assert_allclose(want[:, 1], got1[:50, 1], rtol=0, atol=1e-5)
