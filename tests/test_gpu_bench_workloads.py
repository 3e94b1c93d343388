"""The benchmarked batches themselves, bunch for bunch, against the FP64
oracle (the workloads are built by bench.py's own functions):

* the current scan: all 256 bunches of 256x256 (S log-spaced 0.01..1.5,
  parallel-plates CSR g/R = 0.006, 1000 steps per period) in one batch,
  so the persistent kernel runs with its full grid and the tile chunks of
  the benchmark; the bunches at S = 0.01, 0.3, 0.9 and 1.5 (the last two
  above the bursting threshold, where FP32 and FP64 trajectories part
  exponentially) are compared after every one of the first 10 steps,
  every bunch after 40 steps;
* the oracle builds its own impedance (oracle.make_impedance, FP64) for
  these comparisons: the GPU impedance table is checked against it, and
  the solvers each run on their own;
* the uneven batch: the benchmark's seed, all 96 bunches (meshes
  128..1024, orders 2..4, 2000 steps per period), every bunch after 16
  steps.

Tolerance: the metric's bar, relative L1 of density and profile <= 1e-4
against FP64.
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

import bench
import oracle
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V

pytestmark = pytest.mark.gpu

TOL = 1e-4
THREADS = os.cpu_count() or 1


def rel_l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def oracle_z(p):
    w = P.wake_impedance_args(p)
    return oracle.make_impedance(w["nfreqs"], w["fmax"], w["R_bend"],
                                 w["frev"], w["gap"], w["use_csr"], w["s"],
                                 w["xi"], w["inner_coll_radius"])


def test_full_scan_every_bunch(gpu_ctx):
    p, gap, currents = bench.workload_params()
    n = p["ps_bins"]
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    zo = oracle_z(p)
    zg = z.data()
    assert np.abs(zg - zo).max() <= 1e-6 * np.abs(zo).max()
    batch = bench.make_batch(gpu_ctx, p, currents, z)
    assert batch.cells == 256 * n * n
    descs = [P.fill_desc(oracle.BunchDesc(), p, 0, Ib=float(ib))
             for ib in currents]
    ref = oracle.Sim(descs, Z=zo, dtype=np.float64)
    s_norm = currents / p["I_norm"]
    watch = [int(np.argmin(np.abs(s_norm - s))) for s in (0.01, 0.3, 0.9,
                                                           1.5)]
    for step in range(10):
        batch.step(1)
        ref.step(1, threads=THREADS)
        for i in watch:
            got = batch.density(i)
            err = rel_l1(got, ref.density(i))
            assert err <= TOL, (step, i, s_norm[i], err)
    batch.step(30)
    ref.step(30, threads=THREADS)
    assert gpu_ctx.device_status() == 0
    dens = batch.download().reshape(256, n, n)
    worst = 0.0
    for i in range(256):
        err = rel_l1(dens[i], ref.density(i))
        worst = max(worst, err)
        assert err <= TOL, (i, s_norm[i], err)
        assert rel_l1(batch.profile(i), ref.profile(i)) <= TOL, i
    print("full scan: worst density L1 vs FP64 after 40 steps %.3g" % worst)


def test_uneven_batch_bench_seed(gpu_ctx):
    ps, keys = bench.uneven_workload(4, 96, 2000)
    zs, zo = {}, {}
    for k in keys:
        pk = next(p for p, _ in ps if p["ps_bins"] == k)
        zs[k] = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(pk))
        zo[k] = oracle_z(pk)
    descs = [P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"],
                         impedance=keys.index(p["ps_bins"]), it=it)
             for p, it in ps]
    b = V.BunchBatch(gpu_ctx, descs, [zs[k] for k in keys])
    steps = 16
    b.step(steps)
    assert gpu_ctx.device_status() == 0
    dens = b.download()

    def run(pi):
        p, it = pi
        d = P.fill_desc(oracle.BunchDesc(), p, 0, Ib=p["Ib"], it=it)
        ref = oracle.Sim([d], Z=zo[p["ps_bins"]], dtype=np.float64)
        ref.step(steps)
        return ref

    # one oracle per bunch (their impedances differ by mesh size), on all
    # host cores (the oracle's calls release the interpreter lock)
    with cf.ThreadPoolExecutor(THREADS) as ex:
        refs = list(ex.map(run, ps))
    worst = 0.0
    for i, ((p, it), ref) in enumerate(zip(ps, refs)):
        n = p["ps_bins"]
        off, _ = b.layout(i)
        got = dens[off:off + n * n].reshape(n, n)
        err = rel_l1(got, ref.density(0))
        worst = max(worst, err)
        assert err <= TOL, (i, n, it, err)
        assert rel_l1(b.profile(i), ref.profile(0)) <= TOL, (i, n, it)
    print("uneven batch: worst density L1 vs FP64 after %d steps %.3g"
          % (steps, worst))


def test_batch_sums_against_fp64(gpu_ctx):
    """The batched step sums in FP32 where the plain path uses FP64: the
    bunch profile (Simpson row sums of the new density, FP32 partial sums
    reduced across the row's lanes) and the charge (a compensated FP32 sum
    of the profile, about 48 significant bits).  Bounds against FP64 sums
    of the same data, on the benchmark's scan after 30 steps: profile
    relative L1 <= 1e-6 and largest row error <= 1e-5 of the peak; charge
    within 1e-12 of the FP64 sum of the same profile, and within 1e-6 of
    the FP64 double sum over the density."""
    p, gap, currents = bench.workload_params()
    n = p["ps_bins"]
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    batch = bench.make_batch(gpu_ctx, p, currents, z)
    batch.step(29)
    dens = batch.download().reshape(256, n, n).astype(np.float64)
    profs = [np.asarray(batch.profile(i), np.float64) for i in range(256)]
    # the filling after a step is the charge of the state it started from
    batch.step(1)
    fill = batch.filling()
    ws = np.asarray(oracle.simpson(n, p["axes"][0], p["axes"][1],
                                   np.float32), np.float64)
    worst_l1 = worst_max = worst_q = worst_qd = 0.0
    for i in range(0, 256, 17):
        prof = profs[i]
        ref = dens[i] @ ws
        worst_l1 = max(worst_l1, np.abs(prof - ref).sum() / np.abs(ref).sum())
        worst_max = max(worst_max, np.abs(prof - ref).max() / ref.max())
        q64 = float(prof @ ws)
        worst_q = max(worst_q, abs(fill[i] - q64) / q64)
        worst_qd = max(worst_qd, abs(fill[i] - float(ref @ ws)) / q64)
    print("profile L1 %.3g, max %.3g; charge vs FP64 of the profile %.3g, "
          "of the density %.3g" % (worst_l1, worst_max, worst_q, worst_qd))
    assert worst_l1 <= 1e-6 and worst_max <= 1e-5
    assert worst_q <= 1e-12 and worst_qd <= 1e-6
