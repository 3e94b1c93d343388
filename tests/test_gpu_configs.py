"""The workloads of the benchmark plan as parity cases against the FP64
oracle (synthetic, seeded; the reference's Gaussian start):

* plain single bunch, 256x256, 500 steps per period, free-space CSR,
  S = 0.05, two synchrotron periods, both solver chains;
* bursting regime, 512x512, parallel-plates CSR (gap/R = 0.006) plus a
  resistive wall, 4000 steps per period, S = 1.2, bunch profile, wake and
  CSR power compared every step;
* uneven batch: seeded mesh sizes 128..1024, currents U(0.1, 1.5),
  interpolation orders 2..4, 2000 steps per period, in one batch.

Tolerance: relative L1 <= 1e-4 of density, profile and wake; CSR power
relative difference <= 1e-4.
"""
import numpy as np
import pytest

import oracle
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V
from inovesa_gb300.solver import PlainSolver

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel_l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def oracle_sim(p, chain, Ib, Z, it=None, clamp=False):
    d = P.fill_desc(oracle.BunchDesc(), p, chain, Ib=Ib, it=it, clamp=clamp)
    return oracle.Sim([d], Z=Z, dtype=np.float64)


@pytest.mark.parametrize("chain", [1, 0])
def test_plain_single_bunch(gpu_ctx, chain):
    n, spt = 256, 500
    # damping time of 100 synchrotron periods
    fs = P.derive(GridSize=n, StepsPerTs=spt)["fs"]
    p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=-1.0,
                 S_csr=0.05, DampingTime=100.0 / fs)
    assert abs(p["e1"] - 2.0 / (100 * spt)) < 1e-12
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    clamp = chain == 1
    s = PlainSolver(gpu_ctx, p, chain=chain, wake_impedance=z, it=4,
                    clamp=clamp)
    ref = oracle_sim(p, chain, p["Ib"], z.data(), it=4, clamp=clamp)
    steps = 2 * spt
    for blk in range(4):
        s.step(steps // 4)
        ref.step(steps // 4)
        assert rel_l1(s.density(), ref.density(0)) <= TOL, blk
        assert rel_l1(s.profile(), ref.profile(0)) <= TOL, blk


def test_bursting_csr_every_step(gpu_ctx):
    n, spt = 512, 4000
    p0 = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0)
    gap = 0.006 * p0["R_bend"]
    p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=gap,
                 S_csr=1.2, WallConductivity=5.8e7)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    zr = V.makeImpedance(gpu_ctx, **P.csr_impedance_args(p))
    zrd = zr.data()
    s = PlainSolver(gpu_ctx, p, chain=0, wake_impedance=z, csr_impedance=zr,
                    it=4)
    ref = oracle_sim(p, 0, p["Ib"], z.data(), it=4)
    dq = s.t1.getDelta(0)
    for step in range(16):
        s.step(1, csr=True)
        # the CSR power of the profile that entered this step, on both sides
        power = s.rdtn.getCSRPower()[0]
        _, rpower = oracle.csr(ref.profile(0), zrd, dq, p["fc"],
                               P.C / p["bl"])
        assert abs(power - rpower) <= TOL * abs(rpower), (step, power,
                                                          rpower)
        ref.step(1)
        assert rel_l1(s.profile(), ref.profile(0)) <= TOL, step
        wk = s.wake_field.getWakePotentials()[0]
        assert rel_l1(wk, ref.wake(0)) <= TOL, step
    assert rel_l1(s.density(), ref.density(0)) <= TOL


def test_uneven_batch(gpu_ctx):
    rng = np.random.default_rng(20241)
    spt = 2000
    sizes = rng.choice([128, 256, 512, 1024], size=10)
    currents = rng.uniform(0.1, 1.5, size=10)
    orders = rng.choice([2, 3, 4], size=10)
    z_by_n, zdata = {}, {}
    for n in sorted(set(int(v) for v in sizes)):
        p0 = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                      VacuumGap=0.0318)
        z_by_n[n] = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p0))
        zdata[n] = z_by_n[n].data()
    keys = sorted(z_by_n)
    specs, descs = [], []
    for n, S, it in zip(sizes, currents, orders):
        n, it = int(n), int(it)
        p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                     VacuumGap=0.0318, S_csr=float(S))
        specs.append((p, it))
        descs.append(P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"],
                                 impedance=keys.index(n), it=it))
    b = V.BunchBatch(gpu_ctx, descs, [z_by_n[k] for k in keys])
    steps = 16
    b.step(steps)
    assert gpu_ctx.device_status() == 0
    dens = b.download()
    for i, (p, it) in enumerate(specs):
        n = p["ps_bins"]
        ref = oracle_sim(p, 0, p["Ib"], zdata[n], it=it)
        ref.step(steps)
        off, _ = b.layout(i)
        got = dens[off:off + n * n].reshape(n, n)
        assert rel_l1(got, ref.density(0)) <= TOL, (i, n, it)
        assert rel_l1(b.profile(i), ref.profile(0)) <= TOL, (i, n, it)
