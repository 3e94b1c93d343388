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


def setup(S, gap=0.0318, n=64, spt=200, padding=2.0):
    p = P.derive(GridSize=n, StepsPerTs=spt, padding=padding, VacuumGap=gap,
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


def test_rotation_chain_nearly_stationary():
    """The rotation chain (src/main.cpp rotation loop: rotation with
    clamping, wake kick, Fokker-Planck): one synchrotron period of the
    restated step changes its potential-well state several times less
    than the Gaussian start (the state's own change, about 1e-4 per period,
    is the rotation's interpolation diffusion on this mesh)."""
    p, Z = setup(0.3, gap=0.0318, n=256, spt=1000)
    ws = P.wakescaling_for(p, p["Ib"])
    start, _ = PW.state(p, Z, ws, chain=1)
    change = {}
    for name, data in (("pw", start), ("gauss", None)):
        d = P.fill_desc(oracle.BunchDesc(), p, 1, Ib=p["Ib"], it=4,
                        clamp=True)
        sim = oracle.Sim([d], Z=Z, data=data, dtype=np.float64)
        a = sim.density(0).copy()
        sim.step(p["opts"]["StepsPerTs"], 4)
        b = sim.density(0)
        change[name] = np.abs(b - a).sum() / np.abs(a).sum()
        sim.close()
    assert change["pw"] * 10 < change["gauss"], change


def beam_setup(S=0.5):
    """64-row meshes with free-space CSR, whose wake reaches the next
    buckets; a padded profile of 1024 cells for buckets 0, 1, 3 spaced 64
    cells, and the wake scaling of the reference's current."""
    p, Z = setup(S, gap=-1.0, padding=16.0)
    ws = P.fill_desc(oracle.BunchDesc(), p, 0, Ib=p["Ib"]).wakescaling
    return p, Z, ws


def test_beam_of_one_is_the_bunch_state():
    """A beam of one member is the single bunch's start, bit for bit in
    FP64 (the same wake of the same profile)."""
    p, Z, ws = beam_setup()
    one, ch = PW.beam_states(p, Z, ws, [0], 0, [1.0], iterations=40)
    ref, ch_ref = PW.state(p, Z, ws, iterations=40)
    assert np.array_equal(one[0], ref)
    assert ch[0] == ch_ref


def test_beam_members_feel_each_other():
    """Three members of a beam in buckets 0, 1, 3: the members' states
    differ from their states alone by far more than the iteration's
    floor, every state carries its filling share, and the iteration
    settles."""
    p, Z, ws = beam_setup()
    fills = [0.5, 0.3, 0.2]
    wsx = PW._simpson(64, (p["axes"][1] - p["axes"][0]) / 63)
    wsy = PW._simpson(64, (p["axes"][4] - p["axes"][3]) / 63)
    states, ch = PW.beam_states(p, Z, ws, [0, 1, 3], 64, fills,
                                iterations=150)
    diffs = []
    for m, f in enumerate(fills):
        alone, _ = PW.state(p, Z, ws, iterations=150, fill=f)
        assert abs(np.einsum("xy,x,y->", states[m], wsx, wsy) - f) < 1e-12
        diffs.append(np.abs(states[m] - alone).sum() / np.abs(alone).sum())
    assert min(diffs) > 1e-3 and max(diffs) > 1e-2, diffs
    assert np.all(ch < 1e-10)
