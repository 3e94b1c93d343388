"""Whole solver steps against the FP64 oracle's solver loop.

Tolerance: the metric's bar, relative L1 of the density <= 1e-4 against
FP64, checked after tens to hundreds of steps; profiles and wakes within
the same bound.
"""
import math
import os

import numpy as np
import pytest

import oracle
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V
from inovesa_gb300.solver import PlainSolver

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel_l1(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).sum()
                 / np.abs(np.asarray(b, np.float64)).sum())


def oracle_sim(p, chain, Ib, Z, it=None, clamp=False, data=None):
    d = P.fill_desc(oracle.BunchDesc(), p, chain, Ib=Ib, it=it, clamp=clamp)
    return oracle.Sim([d], Z=Z, data=data, dtype=np.float64)


CASES = [
    # (grid, steps per period, gap, S, chain, it, clamp, renormalize)
    (128, 500, -1.0, 0.05, 0, 4, False, 0),
    (128, 500, -1.0, 0.05, 1, 4, True, 0),
    (128, 1000, 0.0318, 0.8, 0, 3, False, 10),
    (96, 400, 0.0318, 1.2, 1, 2, False, -1),
]


@pytest.mark.parametrize("case", CASES)
def test_plain_loop(gpu_ctx, case):
    n, spt, gap, S, chain, it, clamp, renorm = case
    p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=gap,
                 S_csr=S, RenormalizeCharge=renorm, InterpolationPoints=it)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    s = PlainSolver(gpu_ctx, p, chain=chain, wake_impedance=z, it=it,
                    clamp=clamp)
    ref = oracle_sim(p, chain, p["Ib"], z.data(), it=it, clamp=clamp)
    for block in range(3):
        s.step(40)
        ref.step(40)
        assert rel_l1(s.density(), ref.density(0)) <= TOL, block
        assert rel_l1(s.profile(), ref.profile(0)) <= TOL
    wk = s.wake_field.getWakePotentials()[0]
    assert np.abs(wk - ref.wake(0)).sum() <= TOL * np.abs(ref.wake(0)).sum()


def make_batch(ctx, specs, z_by_n):
    """specs: list of (p, chain, Ib, it, clamp); one impedance per mesh
    size."""
    sizes = sorted(z_by_n)
    descs, zs = [], [z_by_n[k] for k in sizes]
    for p, chain, ib, it, clamp in specs:
        d = P.fill_desc(V.BunchDesc(), p, chain, Ib=ib,
                        impedance=sizes.index(p["ps_bins"]), it=it,
                        clamp=clamp)
        descs.append(d)
    return V.BunchBatch(ctx, descs, zs)


def test_batch_matches_oracle(gpu_ctx):
    specs, z_by_n, zdata = [], {}, {}
    for n in (64, 128):
        p0 = P.derive(GridSize=n, StepsPerTs=500, padding=2.0,
                      VacuumGap=0.0318)
        z_by_n[n] = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p0))
        zdata[n] = z_by_n[n].data()
    for k, (n, chain, it, clamp, S) in enumerate([
            (128, 0, 4, False, 0.05), (128, 0, 4, False, 1.0),
            (64, 0, 3, False, 0.5), (128, 1, 4, True, 0.3),
            (64, 1, 2, False, 0.9), (128, 0, 2, False, 1.4)]):
        p = P.derive(GridSize=n, StepsPerTs=500, padding=2.0,
                     VacuumGap=0.0318, S_csr=S,
                     RenormalizeCharge=(5 if k == 1 else 0))
        specs.append((p, chain, p["Ib"], it, clamp))
    b = make_batch(gpu_ctx, specs, z_by_n)
    refs = [oracle_sim(p, ch, ib, zdata[p["ps_bins"]], it=it, clamp=cl)
            for p, ch, ib, it, cl in specs]
    for blk in range(3):
        b.step(25)
        for r in refs:
            r.step(25)
        dens = b.download()
        for i, r in enumerate(refs):
            off, _ = b.layout(i)
            n = specs[i][0]["ps_bins"]
            got = dens[off:off + n * n].reshape(n, n)
            assert rel_l1(got, r.density(0)) <= TOL, (blk, i)
            assert rel_l1(b.profile(i), r.profile(0)) <= TOL, (blk, i)
    f = b.filling()
    for i, r in enumerate(refs):
        assert abs(f[i] - 1) < 5e-3
    assert gpu_ctx.device_status() == 0


def test_batch_scan_256(gpu_ctx):
    """256^2 meshes at the two ends of the benchmark's current scan, plus a
    few bunches in between so that tiles of several bunches share CTAs."""
    n = 256
    p0 = P.derive(GridSize=n, StepsPerTs=1000, padding=2.0)
    gap = 0.006 * p0["R_bend"]
    p = P.derive(GridSize=n, StepsPerTs=1000, padding=2.0, VacuumGap=gap)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    currents = [0.01, 0.3, 0.9, 1.5]
    specs = [(p, 0, s * p["I_norm"], 4, False) for s in currents]
    b = make_batch(gpu_ctx, specs, {n: z})
    steps = 60
    b.step(steps)
    assert gpu_ctx.device_status() == 0
    dens = b.download()
    zd = z.data()
    for i, s in enumerate(currents):
        ref = oracle_sim(p, 0, s * p["I_norm"], zd)
        ref.step(steps)
        got = dens[i * n * n:(i + 1) * n * n].reshape(n, n)
        assert rel_l1(got, ref.density(0)) <= TOL, (s, rel_l1(got, ref.density(0)))


def test_batch_tilings_agree(gpu_ctx, monkeypatch):
    """Every tiling of the batch gives the same bits: tiles of 4..64 rows,
    short tail tiles, several tiles of different mesh sizes and bunches per
    persistent CTA, both chains in one batch; two bunches against the
    oracle."""
    sizes = (256, 128, 256, 64)
    z_by_n, zdata = {}, {}
    for n in set(sizes):
        p0 = P.derive(GridSize=n, StepsPerTs=1000, padding=2.0,
                      VacuumGap=0.0318)
        z_by_n[n] = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p0))
        zdata[n] = z_by_n[n].data()
    specs = []
    nb = 60
    for k in range(nb):
        n = sizes[k % 4]
        chain = 1 if k % 7 == 3 else 0
        p = P.derive(GridSize=n, StepsPerTs=1000, padding=2.0,
                     VacuumGap=0.0318, S_csr=0.05 + 1.4 * k / (nb - 1),
                     RenormalizeCharge=(3 if k % 5 == 1 else 0))
        specs.append((p, chain, p["Ib"], 4, False))
    steps = 40
    runs = []
    for cells in ("2048", "3072", "6144", "16"):
        monkeypatch.setenv("VFPS_TILE_CELLS", cells)
        b = make_batch(gpu_ctx, specs, z_by_n)
        b.step(steps)
        assert gpu_ctx.device_status() == 0, cells
        runs.append(b.download())
        layout = [b.layout(i) for i in range(nb)]
    assert np.all(np.isfinite(runs[0]))
    for cells, r in zip(("3072", "6144", "16"), runs[1:]):
        assert np.array_equal(r, runs[0]), cells
    for i in (nb - 2, 3):
        p, ch, ib, it, cl = specs[i]
        n = p["ps_bins"]
        ref = oracle_sim(p, ch, ib, zdata[n], it=it, clamp=cl)
        ref.step(steps)
        off, _ = layout[i]
        got = runs[0][off:off + n * n].reshape(n, n)
        assert rel_l1(got, ref.density(0)) <= TOL, i


@pytest.mark.parametrize("n, cells, nb", [(512, "3072", 12),
                                           (256, "1280", 24)])
def test_short_tail_tile_beyond_halo(gpu_ctx, monkeypatch, n, cells, nb):
    """A bunch's last tile shorter than the halo below it (512 rows in
    6-row tiles end in 2 rows, 256 in 5-row tiles in 1; the linear
    interpolation's halo is 3 rows deep): when that tile continues its
    predecessor in one CTA, all of its new staged rows lie beyond the mesh
    end, and the step must stage none of them.  Enough bunches that the
    persistent CTAs walk several tiles each; two of them against the
    oracle."""
    p0 = P.derive(GridSize=n, StepsPerTs=2000, padding=2.0,
                  VacuumGap=0.0318)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p0))
    specs = []
    for k in range(nb):
        p = P.derive(GridSize=n, StepsPerTs=2000, padding=2.0,
                     VacuumGap=0.0318, S_csr=0.2 + 1.2 * k / (nb - 1))
        specs.append((p, 0, p["Ib"], 2, False))
    monkeypatch.setenv("VFPS_TILE_CELLS", cells)
    b = make_batch(gpu_ctx, specs, {n: z})
    steps = 12
    b.step(steps)
    assert gpu_ctx.device_status() == 0
    dens = b.download()
    for i in (0, nb - 1):
        p, ch, ib, it, cl = specs[i]
        ref = oracle_sim(p, ch, ib, z.data(), it=it, clamp=cl)
        ref.step(steps)
        off, _ = b.layout(i)
        got = dens[off:off + n * n].reshape(n, n)
        assert rel_l1(got, ref.density(0)) <= TOL, i


def test_batch_large_shifts(gpu_ctx):
    """Few steps per period (50 on 256-row meshes): kick and drift offsets
    up to 16 cells, so the kick windows of the edge columns reach past the
    8 zero floats left of a staged row (the bounds-checked path) and the
    halos are 17 rows deep (4-row tiles, an 80-slot ring).  Against the
    FP64 oracle."""
    n, spt = 256, 50
    p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=0.0318,
                 S_csr=0.3)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    specs = [(p, 0, p["Ib"], 4, False), (p, 0, 0.5 * p["Ib"], 3, False)]
    b = make_batch(gpu_ctx, specs, {n: z})
    steps = 25
    b.step(steps)
    assert gpu_ctx.device_status() == 0
    dens = b.download()
    for i, (p_, ch, ib, it, cl) in enumerate(specs):
        ref = oracle_sim(p_, ch, ib, z.data(), it=it, clamp=cl)
        ref.step(steps)
        off, _ = b.layout(i)
        got = dens[off:off + n * n].reshape(n, n)
        assert rel_l1(got, ref.density(0)) <= TOL, (i, rel_l1(got, ref.density(0)))


def test_batch_refuses_halos_beyond_shared_memory(gpu_ctx):
    """512-row meshes at 60 steps per period: drift offsets of 27 cells
    make a tile with its halo too deep for the ring in shared memory; the
    batch is refused with an error instead of being launched."""
    n, spt = 512, 60
    p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=0.0318,
                 S_csr=0.3)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    with pytest.raises(V.VfpsError, match="shared memory"):
        make_batch(gpu_ctx, [(p, 0, p["Ib"], 4, False)], {n: z})
    assert gpu_ctx.device_status() == 0


def test_batch_rejects_wider_meshes(gpu_ctx):
    """Batched meshes go up to 1024 rows (the ring kernel); a 2048-row mesh
    is refused with a clear error (the plain path takes it)."""
    p = P.derive(GridSize=2048, StepsPerTs=4000, padding=2.0,
                 VacuumGap=0.0318, S_csr=0.6)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    with pytest.raises(V.InvalidArgument, match="64..1024"):
        make_batch(gpu_ctx, [(p, 0, p["Ib"], 4, False)], {2048: z})
    assert gpu_ctx.device_status() == 0


def test_batch_wide_meshes(gpu_ctx):
    """Meshes of 512 rows (the ring kernel with four column groups per
    lane) and 1024 rows (the tiled chain-0 kernel) next to narrow ones in
    one batch, against the FP64 oracle."""
    specs, z_by_n, zdata = [], {}, {}
    for n in (128, 512, 1024):
        spt = 1000 if n < 1024 else 2000
        p0 = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                      VacuumGap=0.0318)
        z_by_n[n] = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p0))
        zdata[n] = z_by_n[n].data()
    for n, S, it in ((512, 0.4, 4), (128, 0.9, 3), (1024, 1.2, 4),
                     (512, 1.4, 2)):
        spt = 1000 if n < 1024 else 2000
        p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                     VacuumGap=0.0318, S_csr=S)
        specs.append((p, 0, p["Ib"], it, False))
    b = make_batch(gpu_ctx, specs, z_by_n)
    steps = 24
    b.step(steps)
    assert gpu_ctx.device_status() == 0
    dens = b.download()
    for i, (p, ch, ib, it, cl) in enumerate(specs):
        n = p["ps_bins"]
        ref = oracle_sim(p, ch, ib, zdata[n], it=it, clamp=cl)
        ref.step(steps)
        off, _ = b.layout(i)
        got = dens[off:off + n * n].reshape(n, n)
        assert rel_l1(got, ref.density(0)) <= TOL, (i, n)
        assert rel_l1(b.profile(i), ref.profile(0)) <= TOL, (i, n)


def test_batch_equals_plain_loop(gpu_ctx):
    """The fused kernel and the one-map-per-launch loop agree."""
    n = 128
    p = P.derive(GridSize=n, StepsPerTs=500, padding=2.0, VacuumGap=-1.0,
                 S_csr=0.6)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    for chain in (0, 1):
        s = PlainSolver(gpu_ctx, p, chain=chain, wake_impedance=z)
        b = make_batch(gpu_ctx, [(p, chain, p["Ib"], 4, False)], {n: z})
        s.step(64)
        b.step(64)
        assert rel_l1(b.density(0), s.density()) <= 2e-5


def test_batch_run_end_to_end(gpu_ctx):
    n = 64
    p = P.derive(GridSize=n, StepsPerTs=500, padding=2.0, VacuumGap=-1.0,
                 S_csr=0.3)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    b = make_batch(gpu_ctx, [(p, 0, p["Ib"], 4, False)] * 3, {n: z})
    start = b.download()
    b.step(10)
    after10 = b.download()
    out = np.zeros_like(start)
    prof = np.zeros(3 * n, np.float32)
    fill = np.zeros(3, np.float32)
    b.run(start, 10, out, prof, fill)
    # restarting from the same state reproduces the trajectory (the
    # profile of an uploaded state is recomputed from it)
    assert rel_l1(out, after10) <= 1e-6
    assert np.all(np.abs(fill - 1) < 1e-2)
    assert np.all(prof.reshape(3, n).sum(1) > 0)


def test_fast_ring_kernel(gpu_ctx, monkeypatch):
    """The benchmark's lattice (256 rows, 1000 steps per period, centred
    mesh) runs on the fast ring kernel (composite y-kick, sliding-window
    drift); the same batch on the classic ring kernel agrees with it to
    rounding (the two kicks in one stencil; 2e-5 relative L1 after 40
    steps) and both meet the bar against FP64.  A lattice whose drift
    shift changes inside a group of 4 energy columns (50 steps per period)
    stays on the classic kernel."""
    n = 256
    p0 = P.derive(GridSize=n, StepsPerTs=1000, padding=2.0)
    gap = 0.006 * p0["R_bend"]
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(
        P.derive(GridSize=n, StepsPerTs=1000, padding=2.0, VacuumGap=gap)))
    specs = []
    for S in (0.01, 0.2, 0.7, 1.5):
        p = P.derive(GridSize=n, StepsPerTs=1000, padding=2.0,
                     VacuumGap=gap, S_csr=S,
                     RenormalizeCharge=(7 if S == 0.7 else 0))
        specs.append((p, 0, p["Ib"], 4, False))
    steps = 40
    fast = make_batch(gpu_ctx, specs, {n: z})
    tiles = fast.kernel_tiles()
    assert tiles["k_bmaps0f"] > 0 and tiles["k_bmaps0"] == 0, tiles
    fast.step(steps)
    monkeypatch.setenv("VFPS_RING_KERNEL", "classic")
    classic = make_batch(gpu_ctx, specs, {n: z})
    tiles = classic.kernel_tiles()
    assert tiles["k_bmaps0f"] == 0 and tiles["k_bmaps0"] > 0, tiles
    classic.step(steps)
    assert gpu_ctx.device_status() == 0
    a, b = fast.download(), classic.download()
    for i, (p, ch, ib, it, cl) in enumerate(specs):
        off, _ = fast.layout(i)
        ga = a[off:off + n * n].reshape(n, n)
        gb = b[off:off + n * n].reshape(n, n)
        assert rel_l1(ga, gb) <= 2e-5, i
        ref = oracle_sim(p, ch, ib, z.data(), it=it, clamp=cl)
        ref.step(steps)
        assert rel_l1(ga, ref.density(0)) <= TOL, i
        assert rel_l1(fast.profile(i), ref.profile(0)) <= TOL, i
    monkeypatch.delenv("VFPS_RING_KERNEL")
    p = P.derive(GridSize=n, StepsPerTs=50, padding=2.0, VacuumGap=0.0318,
                 S_csr=0.3)
    odd = make_batch(gpu_ctx, [(p, 0, p["Ib"], 4, False)], {n: z})
    tiles = odd.kernel_tiles()
    assert tiles["k_bmaps0f"] == 0 and tiles["k_bmaps0"] > 0, tiles


def test_fast_ring_kernel_512(gpu_ctx, monkeypatch):
    """512-row meshes on the lattices of the bursting and uneven workloads
    (4000 and 2000 steps per period, g/R = 0.006, resistive wall; orders
    2..4) run on the fast ring kernel's half-row form (a pair of warps per
    output row, the halves' row sums joined in shared memory).  Against the
    classic 512-row ring kernel: density and profile within 2e-5 relative
    L1 after 40 steps; against FP64: the bar; the profile against the FP64
    Simpson sums of the same density rows (relative L1 <= 1e-6, largest
    row error <= 1e-5 of the peak)."""
    n = 512
    gap = 0.006 * P.derive(GridSize=n, StepsPerTs=4000, padding=2.0)["R_bend"]
    specs = []
    for spt, S, it in ((4000, 0.8, 4), (4000, 1.6, 4), (2000, 0.3, 2),
                       (2000, 1.2, 3)):
        p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=gap,
                     S_csr=S, WallConductivity=5.8e7)
        specs.append((p, 0, p["Ib"], it, False))
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(specs[0][0]))
    steps = 40
    fast = make_batch(gpu_ctx, specs, {n: z})
    tiles = fast.kernel_tiles()
    assert tiles["k_bmaps0f"] > 0 and tiles["k_bmaps0<4>"] == 0, tiles
    fast.step(steps)
    monkeypatch.setenv("VFPS_RING_KERNEL", "classic")
    classic = make_batch(gpu_ctx, specs, {n: z})
    tiles = classic.kernel_tiles()
    assert tiles["k_bmaps0f"] == 0 and tiles["k_bmaps0<4>"] > 0, tiles
    classic.step(steps)
    monkeypatch.delenv("VFPS_RING_KERNEL")
    assert gpu_ctx.device_status() == 0
    a, b = fast.download(), classic.download()
    ws = np.asarray(oracle.simpson(n, specs[0][0]["axes"][0],
                                   specs[0][0]["axes"][1], np.float32),
                    np.float64)
    for i, (p, ch, ib, it, cl) in enumerate(specs):
        off, _ = fast.layout(i)
        ga = a[off:off + n * n].reshape(n, n)
        gb = b[off:off + n * n].reshape(n, n)
        assert rel_l1(ga, gb) <= 2e-5, i
        assert rel_l1(fast.profile(i), classic.profile(i)) <= 2e-5, i
        sums = ga.astype(np.float64) @ ws
        prof = np.asarray(fast.profile(i), np.float64)
        assert np.abs(prof - sums).sum() / np.abs(sums).sum() <= 1e-6, i
        assert np.abs(prof - sums).max() <= 1e-5 * sums.max(), i
        ref = oracle_sim(p, ch, ib, z.data(), it=it, clamp=cl)
        ref.step(steps)
        assert rel_l1(ga, ref.density(0)) <= TOL, i
        assert rel_l1(fast.profile(i), ref.profile(0)) <= TOL, i


def test_fast_ring_kernel_1024(gpu_ctx, monkeypatch):
    """1024-row meshes on the lattice of the uneven workload (2000 steps per
    period: drift offsets up to 1.6 cells, so some groups of 4 energy
    columns span two drift shifts) and a 4000-step lattice (one shift per
    group), orders 2..4: the fast ring kernel in parts of 256 columns with
    a 5-row drift window.  Against the classic 1024-row kernel (k_bmaps0w):
    density and profile within 2e-5 relative L1 after 24 steps; against
    FP64: the bar; the profile against the FP64 Simpson sums of the
    density rows."""
    n = 1024
    gap = 0.006 * P.derive(GridSize=n, StepsPerTs=2000, padding=2.0)["R_bend"]
    specs = []
    for spt, S, it in ((2000, 0.4, 4), (2000, 1.3, 2), (2000, 0.9, 3),
                       (4000, 1.1, 4)):
        p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=gap,
                     S_csr=S)
        specs.append((p, 0, p["Ib"], it, False))
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(specs[0][0]))
    steps = 24
    fast = make_batch(gpu_ctx, specs, {n: z})
    tiles = fast.kernel_tiles()
    assert tiles["k_bmaps0f"] > 0 and tiles["k_bmaps0w"] == 0, tiles
    fast.step(steps)
    monkeypatch.setenv("VFPS_RING_KERNEL", "classic")
    classic = make_batch(gpu_ctx, specs, {n: z})
    tiles = classic.kernel_tiles()
    assert tiles["k_bmaps0f"] == 0 and tiles["k_bmaps0w"] > 0, tiles
    classic.step(steps)
    monkeypatch.delenv("VFPS_RING_KERNEL")
    assert gpu_ctx.device_status() == 0
    a, b = fast.download(), classic.download()
    ws = np.asarray(oracle.simpson(n, specs[0][0]["axes"][0],
                                   specs[0][0]["axes"][1], np.float32),
                    np.float64)
    for i, (p, ch, ib, it, cl) in enumerate(specs):
        off, _ = fast.layout(i)
        ga = a[off:off + n * n].reshape(n, n)
        gb = b[off:off + n * n].reshape(n, n)
        assert rel_l1(ga, gb) <= 2e-5, i
        assert rel_l1(fast.profile(i), classic.profile(i)) <= 2e-5, i
        sums = ga.astype(np.float64) @ ws
        prof = np.asarray(fast.profile(i), np.float64)
        assert np.abs(prof - sums).sum() / np.abs(sums).sum() <= 1e-6, i
        assert np.abs(prof - sums).max() <= 1e-5 * sums.max(), i
        ref = oracle_sim(p, ch, ib, z.data(), it=it, clamp=cl)
        ref.step(steps, threads=os.cpu_count() or 1)
        assert rel_l1(ga, ref.density(0)) <= TOL, i
        assert rel_l1(fast.profile(i), ref.profile(0)) <= TOL, i


@pytest.mark.parametrize("tile_cells", ["2048", "12288"])
def test_fast_ring_tile_sizes(gpu_ctx, monkeypatch, tile_cells):
    """The fast ring kernel's 512- and 1024-row forms at the smallest and
    largest tile sizes the autotuner tries (4-row tiles, where a group of
    warps walks 2 rows and drops the other 2 of its 4-row step; 24- and
    12-row tiles), a 512- and a 1024-row bunch in one batch: against the
    classic kernels (at their own tiles) after 12 steps (2e-5 relative
    L1)."""
    monkeypatch.setenv("VFPS_TILE_CELLS", tile_cells)
    specs, zs = [], {}
    for n, spt, S, it in ((512, 4000, 1.1, 4), (1024, 2000, 0.7, 3)):
        p0 = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0)
        p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                     VacuumGap=0.006 * p0["R_bend"], S_csr=S)
        specs.append((p, 0, p["Ib"], it, False))
        zs[n] = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    fast = make_batch(gpu_ctx, specs, zs)
    assert fast.kernel_tiles()["k_bmaps0f"] > 0
    fast.step(12)
    # the classic kernels at the autotuner's tiles (12288-cell tiles of a
    # 1024-row mesh do not fit k_bmaps0w's shared memory)
    monkeypatch.delenv("VFPS_TILE_CELLS")
    monkeypatch.setenv("VFPS_RING_KERNEL", "classic")
    classic = make_batch(gpu_ctx, specs, zs)
    assert classic.kernel_tiles()["k_bmaps0f"] == 0
    classic.step(12)
    assert gpu_ctx.device_status() == 0
    for i in range(len(specs)):
        assert rel_l1(fast.density(i), classic.density(i)) <= 2e-5, i
        assert rel_l1(fast.profile(i), classic.profile(i)) <= 2e-5, i
