"""Derived run parameters (inovesa_gb300/params.py, the derivations of
src/main.cpp:163-355 and 593-760 from the options of
src/IO/ProgramOptions.cpp): the shapes the benchmark workloads are quoted
on, the round trip of the normalised current, and the relations between
the derived quantities.  No GPU."""
import math

import pytest

from inovesa_gb300 import params as P


def test_upper_power_of_two():
    # src/HelperFunctions.cpp:178-189
    vals = (0, 1, 2, 3, 5, 8, 9, 511, 512, 513)
    assert [P.upper_power_of_two(v) for v in vals] == \
        [0, 1, 2, 4, 8, 8, 16, 512, 512, 1024]


def test_headline_shapes():
    """256x256 meshes, 1000 steps per synchrotron period, padding 2 (nmax
    512), parallel plates at g/R = 0.006 with R = c / (2 pi f_rev)."""
    p0 = P.derive(GridSize=256, StepsPerTs=1000, padding=2.0)
    assert p0["R_bend"] == pytest.approx(P.C / (2 * math.pi * 9e6))
    gap = 0.006 * p0["R_bend"]
    assert gap == pytest.approx(0.0318, abs=1e-4)
    p = P.derive(GridSize=256, StepsPerTs=1000, padding=2.0, VacuumGap=gap)
    assert p["ps_bins"] == 256
    assert p["padded_bins"] == 512
    assert p["steps"] == 1000
    assert p["angle"] == pytest.approx(2 * math.pi / 1000)
    assert p["dt"] == pytest.approx(1.0 / (p["fs"] * 1000))
    # +-6 sigma mesh, cell size 12 / (n - 1)
    assert p["qmin"] == pytest.approx(-6.0) and p["qmax"] == pytest.approx(6.0)
    z = P.wake_impedance_args(p)
    assert z["nfreqs"] == 512 and z["gap"] == pytest.approx(gap)


def test_padding_rounds_up_to_a_power_of_two():
    p = P.derive(GridSize=96, padding=3.0)
    assert p["padded_bins"] == 512          # ceil(288) -> 512
    q = P.derive(GridSize=96, padding=3.0, RoundPadding=False)
    assert q["padded_bins"] == 288
    r = P.derive(GridSize=64, padding=0.5)  # padding below 1 counts as 1
    assert r["padded_bins"] == 64


@pytest.mark.parametrize("S", [0.01, 0.3, 1.5])
def test_normalised_current_round_trip(S):
    p = P.derive(S_csr=S)
    assert p["S_csr"] == pytest.approx(S, rel=1e-12)
    assert p["Ib"] == pytest.approx(S * p["I_norm"], rel=1e-12)
    # the wake scaling is linear in the current
    assert P.wakescaling_for(p, 2 * p["Ib"]) == \
        pytest.approx(2 * p["wakescaling"], rel=1e-12)


def test_synchrotron_frequency_and_momentum_compaction():
    """A given synchrotron frequency sets alpha0 (and the reverse): the two
    derivations of src/main.cpp agree."""
    p = P.derive()
    q = P.derive(SyncFreq=p["fs"])
    assert q["alpha"][0] == pytest.approx(p["alpha"][0], rel=1e-12)
    assert q["fs"] == pytest.approx(p["fs"], rel=1e-12)
    assert q["bl"] == pytest.approx(p["bl"], rel=1e-12)


def test_damping_and_fokker_planck_strength():
    """e1 = 2 / (fs t_d steps); t_d defaults to E0 / (V0 f_rev); no damping
    time without radiation gives none."""
    p = P.derive(StepsPerTs=500, DampingTime=1e-3)
    assert p["e1"] == pytest.approx(2.0 / (p["fs"] * 1e-3 * 500))
    d = P.derive(StepsPerTs=500)
    assert d["t_damp"] == pytest.approx(d["E0"] / d["V0"] / d["f_rev"])
    # the plain workload's damping of 100 synchrotron periods
    t = P.derive(StepsPerTs=500, DampingTime=100.0 / d["fs"])
    assert t["e1"] == pytest.approx(2.0 / (100 * 500))


def test_steps_per_revolution_overrides_steps_per_period():
    p = P.derive(StepsPerRevolution=10.0)
    assert p["steps"] == pytest.approx(10.0 * p["f_rev"] / p["fs"])
    assert p["revolutionpart"] == pytest.approx(0.1)


def test_bunch_spacing_in_bins():
    """Buckets are 1 / f_RF apart: in mesh bins, n times that spacing over
    the mesh length (in bunch lengths)."""
    p = P.derive(GridSize=128)
    want = round(128 * (1.0 / p["f_RF"]) * P.C / p["bl"] / p["pqsize"])
    assert p["spacing_bins"] == want


def test_unknown_option_rejected():
    with pytest.raises(ValueError):
        P.derive(GridSizee=128)
