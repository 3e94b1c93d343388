"""The plain maps' row-sweep kernels (k_kick_y4, k_kick_x4 and k_fp4 in
inovesa_gb300/csrc/kernels_maps.cu: 16-byte row sweeps, stencils once per
thread, rows staged in shared memory) against the thread-per-cell kernels
(VFPS_PLAIN_KERNEL=cell) on the same input.  The outputs must be
bit-identical: both kick axes, interpolation orders 2..4, offsets inside
the mesh, at its edges and far outside it, two bunches, mesh sides 4..512
(multiples of 4); both Fokker-Planck derivations and all FP types.  A side
that is not a multiple of 4 stays on the thread-per-cell kernels, checked
against the oracle.  The reference's maps: KickMap::apply
(src/SM/KickMap.cpp:221-266), FokkerPlanckMap::apply
(src/SM/FokkerPlanckMap.cpp:170-213)."""
import numpy as np
import pytest

import oracle
from inovesa_gb300 import vfps as V

pytestmark = pytest.mark.gpu

AXES = (-6.0, 6.0, 2e-3, -6.0, 6.0, 6.11e5)
SIDES = [4, 64, 96, 128, 256, 512]


def density(n, nb, seed):
    rng = np.random.default_rng(seed)
    q = np.linspace(-6, 6, n)
    g = np.exp(-0.5 * (q[:, None] ** 2 + (q[None, :] - 0.3) ** 2))
    d = g[None] * (1 + 0.1 * rng.random((nb, n, n)))
    return (d / d.sum()).astype(np.float32)


def pair(ctx, n, d):
    fill = [1.0 / d.shape[0]] * d.shape[0]
    a = V.PhaseSpace(*AXES, ctx, 1, 1, fill, 1.0, d, n=n)
    b = V.PhaseSpace(*AXES, ctx, 1, 1, fill, 1.0, None, n=n)
    return a, b


def kick_offsets(n, count, seed):
    rng = np.random.default_rng(seed)
    off = rng.uniform(-3.5, 3.5, count)
    # far outside the mesh, and shifts at the extremes a valid tap allows
    edge = [-n, n, n / 2 + 0.25, -(n / 2) - 0.5, n / 2 - 1.5, -(n / 2) + 0.75,
            n / 2 - 0.1, -(n / 2) - 2.9]
    off[:len(edge)] = edge[:count]
    return off.astype(np.float32)


def use_cells(monkeypatch, cells):
    if cells:
        monkeypatch.setenv("VFPS_PLAIN_KERNEL", "cell")
    else:
        monkeypatch.delenv("VFPS_PLAIN_KERNEL", raising=False)


def kick(ctx, monkeypatch, n, d, it, axis, off, cells):
    use_cells(monkeypatch, cells)
    a, b = pair(ctx, n, d)
    km = V.KickMap(a, b, it, False, axis)
    km.swapOffset(off)
    km.apply()
    return b.getData()


@pytest.mark.parametrize("n", SIDES)
@pytest.mark.parametrize("axis", [0, 1])
@pytest.mark.parametrize("it", [2, 3, 4])
def test_kick_rows_equal_cells(gpu_ctx, monkeypatch, n, axis, it):
    d = density(n, 2, seed=n + it)
    a, b = pair(gpu_ctx, n, d)
    count = V.KickMap(a, b, it, False, axis).getForce().size
    off = kick_offsets(n, count, seed=10 * n + axis)
    rows = kick(gpu_ctx, monkeypatch, n, d, it, axis, off, False)
    cells = kick(gpu_ctx, monkeypatch, n, d, it, axis, off, True)
    np.testing.assert_array_equal(rows, cells)
    assert np.abs(rows).max() > 0
    assert gpu_ctx.device_status() == 0


@pytest.mark.parametrize("n", SIDES)
@pytest.mark.parametrize("derivation", [3, 4])
@pytest.mark.parametrize("fptype", [0, 1, 2, 3])
def test_fp_rows_equal_cells(gpu_ctx, monkeypatch, n, derivation, fptype):
    d = density(n, 2, seed=n + derivation)
    e1 = 2.0 / (100 * 500) * 50
    out = []
    for cells in (False, True):
        use_cells(monkeypatch, cells)
        a, b = pair(gpu_ctx, n, d)
        V.FokkerPlanckMap(a, b, n, n, fptype, 0, e1, derivation).apply()
        out.append(b.getData())
    np.testing.assert_array_equal(out[0], out[1])
    assert gpu_ctx.device_status() == 0


def test_side_not_multiple_of_4(gpu_ctx, monkeypatch):
    """n = 66: the thread-per-cell kernels, against the float oracle."""
    n = 66
    use_cells(monkeypatch, False)
    d = density(n, 1, seed=3)
    for axis in (0, 1):
        a, b = pair(gpu_ctx, n, d)
        km = V.KickMap(a, b, 4, False, axis)
        off = kick_offsets(n, km.getForce().size, seed=axis)
        km.swapOffset(off)
        km.apply()
        ref = oracle.kick(axis, d, 4, off, dtype=np.float32)
        assert np.max(np.abs(b.getData() - ref)) <= 2e-6 * np.abs(ref).max()
    e1 = 2.0 / (100 * 500) * 50
    a, b = pair(gpu_ctx, n, d)
    V.FokkerPlanckMap(a, b, n, n, 3, 0, e1, 4).apply()
    idx, w = oracle.fp_stencils(n, AXES, e1, 3, 4, dtype=np.float32)
    ref = oracle.fp_apply(d, 4, idx, w, dtype=np.float32)
    assert np.max(np.abs(b.getData() - ref)) <= 2e-6 * np.abs(ref).max()


def test_x_kick_new_offsets(gpu_ctx, monkeypatch):
    """An x-kick map applied, given new offsets and applied again computes
    with the new ones (its stencil table is rebuilt): equal to a fresh map
    with those offsets, bit for bit."""
    use_cells(monkeypatch, False)
    n = 128
    d = density(n, 2, seed=5)
    a, b = pair(gpu_ctx, n, d)
    km = V.KickMap(a, b, 4, False, 0)
    count = km.getForce().size
    km.swapOffset(kick_offsets(n, count, seed=1))
    km.apply()
    off2 = kick_offsets(n, count, seed=2)
    km.swapOffset(off2)
    km.apply()
    again = b.getData()
    a2, b2 = pair(gpu_ctx, n, d)
    fresh = V.KickMap(a2, b2, 4, False, 0)
    fresh.swapOffset(off2)
    fresh.apply()
    np.testing.assert_array_equal(again, b2.getData())
    assert gpu_ctx.device_status() == 0
