"""The potential-well start's CPU restatement (oracle/potential_well_ref.py)
checked against the reference's own step (the oracle's restatement of the
solver loop, src/main.cpp:948-1053): started from the potential-well state
the step leaves the density nearly unchanged, far less than from the
Gaussian start (src/PS/PhaseSpace.cpp:471-484).  Also the fixed point and
the no-wake limit (a matched, unit-spread state).

Sizes: 64 x 64 meshes for the fixed point and the no-wake limit; the
stationarity check needs a resolved mesh (256 x 256, 21 cells per unit of
spread: on coarser meshes the interpolation's own diffusion moves any
start by about 1e-2 per period) and takes a few seconds."""
import numpy as np
import pytest

import oracle
from oracle import potential_well_ref as PW
from inovesa_gb300 import params as P


def setup(S, gap=0.0318, n=64, spt=200):
    p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=gap,
                 S_csr=S)
    w = P.wake_impedance_args(p)
    Z = oracle.make_impedance(w["nfreqs"], w["fmax"], w["R_bend"], w["frev"],
                              w["gap"], w["use_csr"], w["s"], w["xi"],
                              w["inner_coll_radius"])
    return p, Z


def moments(d, p):
    n = p["ps_bins"]
    a = p["axes"]
    q, dq, _ = oracle.ruler(n, a[0], a[1])
    v, dp, _ = oracle.ruler(n, a[3], a[4])
    ws = PW._simpson(n, dq)
    prof = d @ PW._simpson(n, dp)
    eprof = d.T @ ws
    m = lambda ax, pr, w: ((pr * w * ax).sum() / (pr * w).sum(),
                           np.sqrt((pr * w * ax ** 2).sum() / (pr * w).sum()
                                   - ((pr * w * ax).sum() / (pr * w).sum())
                                   ** 2))
    return m(q, prof, ws), m(v, eprof, PW._simpson(n, dp))


def test_no_wake_is_matched_unit_spread():
    p, _ = setup(0.3)
    d, change = PW.state(p, None, 0.0)
    assert change == 0.0
    (mq, sq), (mp, sp) = moments(d, p)
    assert abs(mq) < 1e-3 and abs(mp) < 1e-3
    # the discrete step's invariant differs from the circle by O(angle)
    assert abs(sq - 1.0) < 5e-3 and abs(sp - 1.0) < 5e-3


@pytest.mark.parametrize("S", [0.1, 0.4])
def test_fixed_point_converges(S):
    p, Z = setup(S)
    ws = P.wakescaling_for(p, p["Ib"])
    d, change = PW.state(p, Z, ws, iterations=150)
    assert change < 1e-9
    n = p["ps_bins"]
    a = p["axes"]
    _, dq, _ = oracle.ruler(n, a[0], a[1])
    w = PW._simpson(n, dq)
    assert abs(np.einsum("xy,x,y->", d, w, w) - 1.0) < 1e-12


def test_nearly_stationary_under_the_reference_step():
    """One synchrotron period of the restated reference loop changes the
    potential-well state several times less than the Gaussian start."""
    p, Z = setup(0.3, gap=0.0318, n=256, spt=1000)
    ws = P.wakescaling_for(p, p["Ib"])
    start, _ = PW.state(p, Z, ws)
    change = {}
    for name, data in (("pw", start), ("gauss", None)):
        d = P.fill_desc(oracle.BunchDesc(), p, 0, Ib=p["Ib"])
        sim = oracle.Sim([d], Z=Z, data=data, dtype=np.float64)
        a = sim.density(0).copy()
        sim.step(p["opts"]["StepsPerTs"], 4)
        b = sim.density(0)
        change[name] = np.abs(b - a).sum() / np.abs(a).sum()
        sim.close()
    assert change["pw"] * 5 < change["gauss"], change
