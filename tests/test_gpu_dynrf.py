"""DynamicRFKickMap (src/SM/DynamicRFKickMap.cpp:15-109) on the device:
without noise and modulation it is the static RF kick map; with a
modulation only, the phase of apply i is syncphase + modampl
sin(2 pi modtimeincrement i) and the offsets are the RF kick of that
phase; with noise, phase and amplitude spread as requested and the
sequence is fixed by the seed.

Tolerances: offsets and densities 1e-6 relative (device sin/tan against
the host's); noise moments within 5 standard errors."""
import math

import numpy as np
import pytest

from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V

pytestmark = pytest.mark.gpu


def grids(ctx, n=128):
    p = P.derive(GridSize=n, StepsPerTs=500, padding=2.0)
    a = p["axes"]
    rng = np.random.default_rng(2)
    d = rng.random((n, n)).astype(np.float32)
    g1 = V.PhaseSpace(*a, ctx, 1, 1, [1.0], 1.0, d, n=n)
    g2 = V.PhaseSpace(*a, ctx, 1, 1, [1.0], 1.0, d, n=n)
    return p, g1, g2


@pytest.mark.parametrize("linear", [True, False])
def test_without_noise_equals_static_map(gpu_ctx, linear):
    p, g1, g2 = grids(gpu_ctx)
    o1 = g1.copy()
    o2 = g2.copy()
    if linear:
        st = V.RFKickMap(g1, o1, p["angle"], p["f_RF"], 4, False)
        dy = V.DynamicRFKickMap(g2, o2, p["angle"], p["revolutionpart"],
                                p["f_RF"], 0.0, 0.0, 0.0, 0.0, 16, 4, False)
    else:
        st = V.RFKickMap.sinusoidal(g1, o1, p["revolutionpart"], p["V_eff"],
                                    p["f_RF"], p["V0"], 4, False)
        dy = V.DynamicRFKickMap.sinusoidal(
            g2, o2, p["revolutionpart"], p["V_eff"], p["f_RF"], p["V0"],
            0.0, 0.0, 0.0, 0.0, 16, 4, False)
    st.apply()
    dy.apply()
    f1, f2 = st.getForce(), dy.getForce()
    assert np.allclose(f2, f1, rtol=1e-6, atol=1e-6 * np.abs(f1).max())
    a, b = o1.getData(), o2.getData()
    assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max()
    mod = dy.getPastModulation()
    assert mod.shape == (1, 2) and mod[0, 1] == 1.0


def test_modulation_only(gpu_ctx):
    p, g1, g2 = grids(gpu_ctx)
    o2 = g2.copy()
    modampl, inc = 0.05, 0.013
    dy = V.DynamicRFKickMap(g2, o2, p["angle"], p["revolutionpart"],
                            p["f_RF"], 0.0, 0.0, modampl, inc, 64, 4, False)
    for _ in range(40):
        dy.apply()
    mod = dy.getPastModulation()
    want = modampl * np.sin(2 * math.pi * inc * np.arange(40))
    assert np.allclose(mod[:, 0], want, atol=1e-6)
    assert np.all(mod[:, 1] == 1.0)
    # offsets of the last apply: the linear RF kick at that phase
    # (src/SM/RFKickMap.cpp:59-68)
    ax = g2.getAxis(0)
    dq, zb = g2.getDelta(0), g2.zerobin(0)
    bl2phase = np.float32(p["bl2phase"])
    ta = np.tan(np.float32(p["angle"]))
    x = np.arange(ax.size, dtype=np.float32)
    off = (ta * (zb - x) + ta * (0 - mod[-1, 0]) / bl2phase / dq) * 1.0
    f = dy.getForce()
    assert np.allclose(f, off, rtol=1e-5, atol=1e-5 * np.abs(off).max())


def test_noise_statistics_and_seed(gpu_ctx):
    p, g1, g2 = grids(gpu_ctx, n=64)
    rp = p["revolutionpart"]
    ps_, as_ = 0.01 * math.sqrt(rp), 0.002 * math.sqrt(rp)
    N = 4000
    runs = []
    for seed in (1, 1, 2):
        o = g2.copy()
        dy = V.DynamicRFKickMap(g2, o, p["angle"], rp, p["f_RF"], ps_, as_,
                                0.0, 0.0, N, 4, False, seed=seed)
        for _ in range(N):
            dy.apply()
        runs.append(dy.getPastModulation())
    m = runs[0]
    for col, sd in ((0, 0.01), (1, 0.002)):
        v = m[:, col] - (1.0 if col else 0.0)
        assert abs(v.mean()) <= 5 * sd / math.sqrt(N)
        assert abs(v.std() - sd) <= 5 * sd / math.sqrt(2 * N)
    assert abs(np.corrcoef(m[:, 0], m[:, 1])[0, 1]) < 0.1
    assert np.array_equal(runs[0], runs[1])
    assert not np.array_equal(runs[0], runs[2])


def test_particles_follow_the_dynamic_kick(gpu_ctx):
    """applyTo of a dynamic map uses the offsets of its last apply (the
    reference's KickMap::applyTo, src/SM/KickMap.cpp:280-303)."""
    p, g1, g2 = grids(gpu_ctx)
    o1, o2 = g1.copy(), g2.copy()
    st = V.RFKickMap(g1, o1, p["angle"], p["f_RF"], 4, False)
    dy = V.DynamicRFKickMap(g2, o2, p["angle"], p["revolutionpart"],
                            p["f_RF"], 0.0, 0.0, 0.0, 0.0, 4, 4, False)
    st.apply()
    dy.apply()
    rng = np.random.default_rng(5)
    pts = rng.uniform(10, 110, size=(50, 2)).astype(np.float32)
    a = st.applyToAll(pts)
    b = dy.applyToAll(pts)
    assert np.allclose(a, b, rtol=0, atol=1e-4)
    assert np.abs(a - pts).max() > 0
