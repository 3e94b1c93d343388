"""vfps_batch_potential_well on the device against its FP64 restatement
(oracle/potential_well_ref.py), through the C ABI.

Tolerance: relative L1 of each density <= 1e-4 (FP32 kernel, FP32 exp,
against FP64); fixed-point change <= 1e-5 (the FP32 floor of the mixing
iteration); bunches of the rotation chain against the restatement's
rotation-chain state.  Then
the device's own solver step: one synchrotron period from the
potential-well state moves the profile at least five times less than
from the Gaussian start."""
import numpy as np
import pytest

from oracle import potential_well_ref as PW
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V
from inovesa_gb300 import warmstart as WS

pytestmark = pytest.mark.gpu


def rel_l1(a, b):
    b = np.asarray(b, np.float64)
    return float(np.abs(np.asarray(a, np.float64) - b).sum()
                 / np.abs(b).sum())


# (mesh, S, gap ratio, chain, wake)
CASES = [(256, 0.10, 0.004, 0, True), (256, 0.40, 0.008, 0, True),
         (128, 0.30, 0.006, 0, True), (256, 0.20, 0.006, 0, False),
         (128, 0.25, 0.006, 1, True)]


def batch(ctx, cases, spt=1000):
    zs, keys, descs, ps = {}, [], [], []
    for n, S, g, chain, wake in cases:
        p = WS.bunch_params(n, spt, S, g, 10.0)
        k = (n, round(g, 9))
        if k not in zs:
            zs[k] = V.makeImpedance(ctx, **P.wake_impedance_args(p))
            keys.append(k)
        d = P.fill_desc(V.BunchDesc(), p, chain,
                        Ib=p["Ib"] if wake else 0.0,
                        impedance=keys.index(k))
        descs.append(d)
        ps.append((p, zs[k].data() if wake else None,
                   d.wakescaling))
    return V.BunchBatch(ctx, descs, [zs[k] for k in keys]), ps


def test_matches_restatement(gpu_ctx):
    b, ps = batch(gpu_ctx, CASES)
    change = b.potential_well(iterations=200, mix=0.5)
    fill = b.filling()
    for i, (n, S, g, chain, wake) in enumerate(CASES):
        got = b.density(i)
        p, Z, ws = ps[i]
        want, _ = PW.state(p, Z, ws, iterations=200, mix=0.5, chain=chain)
        assert rel_l1(got, want) <= 1e-4, (i, rel_l1(got, want))
        assert change[i] <= 1e-5 if wake else change[i] == 0.0
        assert abs(fill[i] - 1.0) < 1e-5
        assert rel_l1(b.profile(i), want @ PW._simpson(
            n, (p["axes"][4] - p["axes"][3]) / (n - 1))) <= 1e-4
    assert gpu_ctx.device_status() == 0


def test_rejects_bad_mixing(gpu_ctx):
    b, _ = batch(gpu_ctx, CASES[:1])
    for mix in (0.0, -0.5, 1.5, float("nan")):
        with pytest.raises(V.VfpsError):
            b.potential_well(10, mix)


def test_nearly_stationary_under_the_solver(gpu_ctx):
    cases = CASES[:2]
    spt = 1000
    change = {}
    for name in ("pw", "gauss"):
        b, _ = batch(gpu_ctx, cases, spt)
        if name == "pw":
            b.potential_well()
        a = np.stack([b.profile(i) for i in range(len(cases))])
        b.step(spt)
        c = np.stack([b.profile(i) for i in range(len(cases))])
        change[name] = np.abs(c - a).sum(1) / np.abs(a).sum(1)
    assert np.all(change["pw"] * 5 < change["gauss"]), change


def test_coupled_beam_matches_restatement(gpu_ctx):
    """A three-bunch beam (buckets 0, 1, 3 spaced 64 cells, free-space CSR
    whose wake reaches the next buckets, filling shares 0.5/0.3/0.2) next
    to a bunch on its own: every member's start against the beam
    restatement (oracle.potential_well_ref.beam_states, the members'
    fields of the previous iteration in each wake), the lone bunch against
    its own; relative L1 <= 1e-4 as above.  The members' states differ
    from their states alone by more than 1e-3, so the check sees the
    coupling."""
    p = P.derive(GridSize=64, StepsPerTs=200, padding=16.0, VacuumGap=-1.0,
                 S_csr=0.5)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    descs = [P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"], impedance=0)
             for _ in range(4)]
    b = V.BunchBatch(gpu_ctx, descs, [z])
    fills = [0.5, 0.3, 0.2]
    b.set_beams([1, 1, 1, 0], [0, 1, 3, 0], 64, fills + [1.0])
    change = b.potential_well(iterations=150, mix=0.5)
    ws = float(np.float32(descs[0].wakescaling))
    want, _ = PW.beam_states(p, z.data(), ws, [0, 1, 3], 64, fills,
                             iterations=150, mix=0.5)
    for m in range(3):
        got = b.density(m)
        assert rel_l1(got, want[m]) <= 1e-4, (m, rel_l1(got, want[m]))
        alone, _ = PW.state(p, z.data(), ws, iterations=150, fill=fills[m])
        assert rel_l1(want[m], alone) > 1e-3
        assert change[m] <= 1e-5
    lone, _ = PW.state(p, z.data(), ws, iterations=150)
    assert rel_l1(b.density(3), lone) <= 1e-4
    assert np.allclose(b.filling(), fills + [1.0], rtol=1e-5)
    assert gpu_ctx.device_status() == 0
