"""CSR power recorded by the batched step (vfps_batch_set_csr) against the
FP64 oracle's updateCSR (src/PS/ElectricField.cpp:133-184) of the same
profiles, and against the plain ElectricField; the ring keeps the steps in
order.

Tolerance: relative 1e-4 of the power (the batch evaluates the spectrum
sum as a quadratic form in FP32; with the shielded impedance its terms
cancel by about 1e3, which leaves errors near 1e-5)."""
import numpy as np
import pytest

import oracle
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V

pytestmark = pytest.mark.gpu

# (mesh, S, gap): shielded and free-space CSR, three mesh sizes (the
# 512-row mesh's wake is summed in blocks by several CTAs)
CASES = [(256, 0.3, 0.0318), (256, 1.0, 0.0318), (128, 0.5, -1.0),
         (256, 0.1, -1.0), (512, 0.6, 0.0318)]


def build(ctx, spt=500):
    zw, zc, ps, descs = [], [], [], []
    for n, S, gap in CASES:
        p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=gap,
                     S_csr=S)
        zw.append(V.makeImpedance(ctx, **P.wake_impedance_args(p)))
        zc.append(V.makeImpedance(ctx, **P.csr_impedance_args(p)))
        ps.append(p)
        descs.append(P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"],
                                 impedance=len(descs)))
    b = V.BunchBatch(ctx, descs, zw)
    return b, ps, zc


def test_csr_power_matches_oracle(gpu_ctx):
    b, ps, zc = build(gpu_ctx)
    nb = len(CASES)
    b.set_csr(zc, list(range(nb)), [p["fc"] for p in ps],
              [P.C / p["bl"] for p in ps], every=1, capacity=4)
    lay = [b.layout(i) for i in range(nb)]
    for s in range(6):
        pr = b.profiles()
        b.step(1)
        steps, power = b.csr()
        assert steps[-1] == s and len(steps) == min(s + 1, 4)
        for i, (n, S, gap) in enumerate(CASES):
            p = ps[i]
            prof = pr[lay[i][1]:lay[i][1] + n]
            dq = (p["axes"][1] - p["axes"][0]) / (n - 1)
            _, ref = oracle.csr(prof, zc[i].data(), np.float32(dq), p["fc"],
                                P.C / p["bl"])
            assert abs(power[-1, i] - ref) <= 1e-4 * abs(ref), (s, i)
    assert gpu_ctx.device_status() == 0


def test_csr_every_and_ring(gpu_ctx):
    b, ps, zc = build(gpu_ctx)
    nb = len(CASES)
    # bunch 1 without CSR; record every third step into 3 slots
    b.set_csr(zc, [0, -1, 2, 3, 4], [p["fc"] for p in ps],
              [P.C / p["bl"] for p in ps], every=3, capacity=3)
    b.step(14)
    steps, power = b.csr()
    assert steps.tolist() == [6, 9, 12]
    assert np.all(power[:, 1] == 0) and np.all(power[:, [0, 2, 3, 4]] > 0)
    b.step(1)     # step 14: not recorded
    steps2, _ = b.csr()
    assert steps2.tolist() == [6, 9, 12]
    # step 15 against the plain ElectricField of the state it starts from
    b.set_csr(zc, [0, 1, 2, 3, 4], [p["fc"] for p in ps],
              [P.C / p["bl"] for p in ps], every=1, capacity=2)
    n, p = CASES[0][0], ps[0]
    d = b.density(0).copy()
    b.step(1)
    steps3, power3 = b.csr()
    assert steps3.tolist() == [15]
    ph = V.PhaseSpace(*p["axes"], gpu_ctx, 1, 1, [1.0], 1.0, d[None], n=n)
    ph.updateXProjection()
    rd = V.ElectricField(ph, zc[0], [0], 0, gpu_ctx, p["f_rev"],
                         p["revolutionpart"])
    rd.updateCSR(p["fc"])
    plain = rd.getCSRPower()[0]
    assert abs(power3[0, 0] - plain) <= 1e-4 * abs(plain)
    # switching off
    b.set_csr([], [-1] * nb, [0.0] * nb, [1.0] * nb, every=0)
    with pytest.raises(V.VfpsError):
        b.csr()
