"""Multi-bunch beams in the batch (vfps_batch_set_beams): the wake of each
member carries the other members' fields at their bucket distances, as the
reference's shared padded profile gives (src/PS/ElectricField.cpp:186-263,
bunch filling src/main.cpp:248-321).

Checks: one step's wake against the oracle's coupled wake of the same
profiles (1e-5 of the largest |wake|, the FP32 Toeplitz sum against the
FFT), on 64-row meshes and on 512-row meshes (rows summed in blocks by
several CTAs per bunch); 40 steps of a three-bunch beam against the plain one-map-per-launch
loop over a three-bunch phase space (density L1 <= 1e-4, the metric's bar);
a bunch outside the beam is unaffected by it; inconsistent beams are
rejected."""
import numpy as np
import pytest

import oracle
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V
from inovesa_gb300.solver import PlainSolver

pytestmark = pytest.mark.gpu

N, SPT = 64, 500
BUCKETS = [0, 1, 3]
SPACING = 70         # buckets close enough that the fields reach across
FILL = [0.5, 0.3, 0.2]


def setup(ctx, extra_alone=True, Ib_alone=None):
    p = P.derive(GridSize=N, StepsPerTs=SPT, padding=16.0, VacuumGap=0.0318,
                 S_csr=0.5)
    z = V.makeImpedance(ctx, **P.wake_impedance_args(p))
    descs = [P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"], impedance=0)
             for _ in BUCKETS]
    if extra_alone:
        descs.append(P.fill_desc(V.BunchDesc(), p, 0,
                                 Ib=Ib_alone or p["Ib"], impedance=0))
    return p, z, V.BunchBatch(ctx, descs, [z])


def rel_l1(a, b):
    b = np.asarray(b, np.float64)
    return float(np.abs(np.asarray(a, np.float64) - b).sum()
                 / np.abs(b).sum())


# (mesh, padding, bucket spacing): one block of rows per bunch, and 512-row
# meshes whose wake is summed by several CTAs per bunch
WAKE_CASES = [(N, 16.0, SPACING), (512, 4.0, 500)]


@pytest.mark.parametrize("n, padding, spacing", WAKE_CASES)
def test_coupled_wake_matches_oracle(gpu_ctx, n, padding, spacing):
    p = P.derive(GridSize=n, StepsPerTs=SPT, padding=padding,
                 VacuumGap=0.0318, S_csr=0.5)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    descs = [P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"], impedance=0)
             for _ in range(4)]
    b = V.BunchBatch(gpu_ctx, descs, [z])
    b.set_beams([1, 1, 1, 0], BUCKETS + [0], spacing, FILL + [1.0])
    lay = [b.layout(i) for i in range(4)]
    pr = b.profiles()
    prof = np.stack([pr[lay[i][1]:lay[i][1] + n] for i in range(4)])
    assert np.allclose(b.filling()[:3], FILL, rtol=1e-5)
    b.step(1)
    wk = b.wake()
    got = np.stack([wk[lay[i][1]:lay[i][1] + n] for i in range(4)])
    ws = float(np.float32(b.descs[0].wakescaling))
    ref = oracle.wake_potential(prof[:3], z.data(), ws, buckets=BUCKETS,
                                spacing=spacing)
    assert np.abs(got[:3] - ref).max() <= 1e-5 * np.abs(ref).max()
    alone = oracle.wake_potential(prof[3:], z.data(), ws)[0]
    assert np.abs(got[3] - alone).max() <= 1e-5 * np.abs(alone).max()
    # the coupling is there: each member alone has another wake
    own = [oracle.wake_potential(prof[i:i + 1], z.data(), ws)[0]
           for i in range(3)]
    assert max(np.abs(own[i] - ref[i]).max() / np.abs(ref[i]).max()
               for i in range(3)) > 1e-3
    assert gpu_ctx.device_status() == 0


def test_beam_matches_plain_loop(gpu_ctx):
    p, z, b = setup(gpu_ctx)
    b.set_beams([1, 1, 1, 0], BUCKETS + [0], SPACING, FILL + [1.0])
    plain = PlainSolver(gpu_ctx, p, chain=0, Ib=p["Ib"], wake_impedance=z,
                        fillings=FILL, buckets=BUCKETS, spacing=SPACING)
    # the same bunch outside any beam, alone in its own batch
    _, _, single = setup(gpu_ctx, extra_alone=False)
    single.set_beams([0, 0, 0], [0, 0, 0], 0, [1.0, 1.0, 1.0])
    for block in range(2):
        b.step(20)
        plain.step(20)
        single.step(20)
        for i in range(3):
            assert rel_l1(b.density(i), plain.density(i)) <= 1e-4, (block, i)
        assert rel_l1(b.density(3), single.density(0)) <= 1e-6
    assert gpu_ctx.device_status() == 0


def test_rejects_inconsistent_beams(gpu_ctx):
    p, z, b = setup(gpu_ctx, Ib_alone=0.5 * P.derive(
        GridSize=N, StepsPerTs=SPT, padding=16.0, VacuumGap=0.0318,
        S_csr=0.5)["Ib"])
    # bunch 3 has another wake scaling: it cannot join the beam
    with pytest.raises(V.VfpsError):
        b.set_beams([1, 1, 1, 1], [0, 1, 3, 4], SPACING)
    with pytest.raises(V.VfpsError):
        b.set_beams([1, 1, 1, 0], BUCKETS + [0], SPACING,
                    [0.5, -0.3, 0.2, 1.0])
    b.set_beams([1, 1, 1, 0], BUCKETS + [0], SPACING)
    with pytest.raises(V.VfpsError):
        b.set_wake_mode(1)   # the tensor-core sum has no coupling
