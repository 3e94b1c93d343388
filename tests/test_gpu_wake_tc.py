"""Wake potentials of a batch on the tensor cores (TF32 split into three
products, FP32 accumulation) against the CUDA-core Toeplitz sum on the same
state, against the FP64 wake of the same profiles, and through a solver run
against the FP64 oracle.

Tolerances: the error against the FP64 product of the same profiles, per
bunch relative to its largest wake value, is at most 2.5e-5 for meshes up
to 256 rows (growing as the square root of the mesh size beyond: FP32
accumulation over n source cells) and within 4x of the CUDA-core FP32
sum's (the Toeplitz sum cancels: its terms are up to ten times the
result); solver densities, relative L1 <= 1e-4.
"""
import numpy as np
import pytest

import oracle
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V

pytestmark = pytest.mark.gpu


def rel_l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def scan_batch(ctx, counts):
    """counts: {n: number of bunches}; currents spread over S 0.05..1.4"""
    zs, zdata, specs, descs = {}, {}, [], []
    keys = sorted(counts)
    for n in keys:
        p0 = P.derive(GridSize=n, StepsPerTs=1000, padding=2.0,
                      VacuumGap=0.0318)
        zs[n] = V.makeImpedance(ctx, **P.wake_impedance_args(p0))
        zdata[n] = zs[n].data()
    for n in keys:
        for S in np.linspace(0.05, 1.4, counts[n]):
            p = P.derive(GridSize=n, StepsPerTs=1000, padding=2.0,
                         VacuumGap=0.0318, S_csr=float(S))
            specs.append(p)
            descs.append(P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"],
                                     impedance=keys.index(n)))
    b = V.BunchBatch(ctx, descs, [zs[k] for k in keys])
    return b, specs, zdata


# 70 bunches of 256 rows (five tiles of 16, the last with 6) and 3 of
# 128; 1024-row meshes (three chunks of the Toeplitz operand in flight,
# all 32 profile chunks staged) next to 64-row ones (two chunks, fewer than
# the stages); 512 rows (five in flight)
WAKE_TC_MIXES = [{256: 70, 128: 3}, {1024: 5, 64: 17}, {512: 20}]


@pytest.mark.parametrize("counts", WAKE_TC_MIXES)
def test_wake_tc_matches_cuda_cores_and_fp64(gpu_ctx, counts):
    # two identical batches reach the same state, then one step each with
    # the wake on the CUDA cores and on the tensor cores
    b0, specs, zdata = scan_batch(gpu_ctx, counts)
    b1, _, _ = scan_batch(gpu_ctx, counts)
    b0.step(30)
    b1.step(30)
    prof = b0.profiles()
    assert np.array_equal(prof, b1.profiles())
    b1.set_wake_mode(1)
    b0.step(1)
    b1.step(1)
    w0, w1 = b0.wake(), b1.wake()
    assert gpu_ctx.device_status() == 0
    # error of both against the FP64 Toeplitz product of the same profiles,
    # relative to the largest wake value of each bunch
    e_cc, e_tc = 0.0, 0.0
    for i, p in enumerate(specs):
        n = p["ps_bins"]
        _, off = b0.layout(i)
        ref = oracle.wake_potential(prof[off:off + n], zdata[n],
                                    float(np.float32(p["wakescaling"])))[0]
        m = np.abs(ref).max()
        e_cc = max(e_cc, np.abs(w0[off:off + n] - ref).max() / m)
        e_tc = max(e_tc, np.abs(w1[off:off + n] - ref).max() / m)
    print("wake error vs FP64 (max over bunches, relative to max |wake|):"
          " CUDA cores %.2e, tensor cores %.2e" % (e_cc, e_tc))
    # FP32 accumulation over K = n source cells: the bound grows as sqrt(n)
    bound = 2.5e-5 * max(1.0, np.sqrt(max(counts) / 256.0))
    assert e_tc <= bound, (e_tc, bound)
    assert e_tc <= 4 * e_cc + 1e-6, (e_tc, e_cc)


def test_wake_tc_solver_run(gpu_ctx):
    b, specs, zdata = scan_batch(gpu_ctx, {256: 6, 128: 2})
    b.set_wake_mode(1)
    steps = 40
    b.step(steps)
    assert gpu_ctx.device_status() == 0
    dens = b.download()
    for i, p in enumerate(specs):
        n = p["ps_bins"]
        d = P.fill_desc(oracle.BunchDesc(), p, 0, Ib=p["Ib"])
        ref = oracle.Sim([d], Z=zdata[n], dtype=np.float64)
        ref.step(steps)
        off, _ = b.layout(i)
        got = dens[off:off + n * n].reshape(n, n)
        assert rel_l1(got, ref.density(0)) <= 1e-4, (i, n)
