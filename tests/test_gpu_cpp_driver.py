"""The C++ driver (the reference's solver loop over include/vfps.hpp)
against the Python mirror of the same loop and against the FP64 oracle.
Both host programs make the same C-ABI calls in the same order, so their
densities agree to float rounding (<= 1e-6 relative L1); against FP64 the
metric's bar, relative L1 <= 1e-4."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from inovesa_gb300 import build as B
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V
from inovesa_gb300.solver import PlainSolver

pytestmark = pytest.mark.gpu


def rel_l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).sum() / np.abs(b).sum())


@pytest.mark.parametrize("chain,clamp,csr", [(0, False, True),
                                             (1, True, False)])
def test_cpp_driver(gpu_ctx, tmp_path, chain, clamp, csr):
    n, steps = 128, 150
    p = P.derive(GridSize=n, StepsPerTs=500, padding=2.0, VacuumGap=0.0318,
                 S_csr=0.6)
    rf = tmp_path / "run.txt"
    rf.write_text(P.run_file(p, chain=chain, it=4, clamp=clamp,
                             steps=steps, csr=csr))
    exe = B.build_driver()
    out = str(tmp_path / "out")
    r = subprocess.run([exe, str(rf), out], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    dens = np.fromfile(out + ".density", np.float32).reshape(n, n)
    prof = np.fromfile(out + ".profile", np.float32)

    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    zr = V.makeImpedance(gpu_ctx, **P.csr_impedance_args(p)) if csr else None
    s = PlainSolver(gpu_ctx, p, chain=chain, wake_impedance=z,
                    csr_impedance=zr, it=4, clamp=clamp)
    power = []
    for _ in range(steps):
        s.step(1, csr=csr)
        if csr:
            power.append(s.rdtn.getCSRPower()[0])
    assert rel_l1(dens, s.density()) <= 1e-6
    assert rel_l1(prof, s.profile()) <= 1e-6
    if csr:
        cp = np.loadtxt(out + ".csr")
        assert cp.shape == (steps,)
        assert np.allclose(cp, power, rtol=1e-6, atol=0)

    d = P.fill_desc(oracle.BunchDesc(), p, chain, Ib=p["Ib"], it=4,
                    clamp=clamp)
    ref = oracle.Sim([d], Z=z.data(), dtype=np.float64)
    ref.step(steps)
    assert rel_l1(dens, ref.density(0)) <= 1e-4
