"""Resume through the run directory: N steps, save, a new solver from the
saved phase space, N more steps equals 2N uninterrupted steps bit for bit
(both chains, with renormalisation on a schedule that straddles the
restart)."""
import numpy as np
import pytest

from inovesa_gb300 import params as P
from inovesa_gb300 import record as R
from inovesa_gb300 import vfps as V
from inovesa_gb300.solver import PlainSolver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("chain", [0, 1])
def test_resume_continues_bit_for_bit(gpu_ctx, tmp_path, chain):
    n, N = 128, 37
    p = P.derive(GridSize=n, StepsPerTs=500, padding=2.0, VacuumGap=0.0318,
                 S_csr=0.7, RenormalizeCharge=10)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    zr = V.makeImpedance(gpu_ctx, **P.csr_impedance_args(p))
    full = PlainSolver(gpu_ctx, p, chain=chain, wake_impedance=z, it=4)
    full.step(2 * N)

    first = PlainSolver(gpu_ctx, p, chain=chain, wake_impedance=z,
                        csr_impedance=zr, it=4)
    rec = R.Recorder(str(tmp_path), first.t1.getAxis(0),
                     first.t1.getAxis(1))
    first.step(N, csr=True)
    R.record_plain(rec, first, N * p["dt"], csr=True)
    rec.close()
    state, t = R.resume_state(str(tmp_path))
    assert abs(t - N * p["dt"]) < 1e-15
    second = PlainSolver(gpu_ctx, p, chain=chain, wake_impedance=z, it=4,
                         data=state, resume_step=N)
    second.step(N)
    assert np.array_equal(second.density(), full.density())
    # the recorded profile is the state's projection
    prof = R.read(str(tmp_path), "/BunchProfile/data")[0, 0]
    assert np.allclose(prof, first.profile(), rtol=0, atol=0)
