"""Derived simulation parameters, as the reference solver computes them
from its options (src/main.cpp:163-355, 593-760), and the per-bunch
descriptors the batched C ABI takes.

Defaults are the reference's option defaults
(src/IO/ProgramOptions.cpp:29-268).  The "normalised current" S of a
configuration is S_csr = Ib / I_norm with I_norm from src/main.cpp:386-388.
"""
import math

C = 2.99792458e8            # inc/defines.hpp:48
EPS0 = 8.854187817e-12      # inc/defines.hpp:51
E_CHARGE = 1.602e-19        # inc/defines.hpp:57
I_ALFVEN = 17045.0          # inc/defines.hpp:60
ME_EV = 510998.9            # inc/defines.hpp:63

DEFAULTS = dict(
    GridSize=256, PhaseSpaceSize=12.0, PhaseSpaceShiftX=0.0,
    PhaseSpaceShiftY=0.0, BeamEnergySpread=4.7e-4, BeamEnergy=1.3e9,
    BendingRadius=-1.0, RevolutionFrequency=9e6, CutoffFreq=23e9,
    HarmonicNumber=50.0, VacuumGap=0.03, AcceleratingVoltage=1e6,
    LinearRF=True, SyncFreq=0.0, alpha0=4e-3, alpha1=0.0, alpha2=0.0,
    BunchCurrent=(1e-3,), InitialDistZoom=1.0, StepsPerTs=1000,
    StepsPerRevolution=0.0, rotations=5.0, DampingTime=-1.0, padding=8.0,
    RoundPadding=True, WallConductivity=0.0, WallSusceptibility=0.0,
    CollimatorRadius=0.0, UseCSR=True, FPType=3, FPTrack=3, derivation=4,
    InterpolationPoints=4, InterpolateClamped=False, RenormalizeCharge=0,
)


def upper_power_of_two(v):
    """src/HelperFunctions.cpp:178-189."""
    v = int(v)
    if v <= 1:
        return 1 if v == 1 else 0
    return 1 << (v - 1).bit_length()


def derive(**kw):
    """All quantities main.cpp derives from the options."""
    o = dict(DEFAULTS)
    unknown = set(kw) - set(DEFAULTS) - {"S_csr"}
    if unknown:
        raise ValueError("unknown options: %s" % sorted(unknown))
    o.update({k: v for k, v in kw.items() if k != "S_csr"})
    p = dict(opts=o)
    ps_bins = int(o["GridSize"])
    pqsize = float(o["PhaseSpaceSize"])
    qcenter = -o["PhaseSpaceShiftX"] * pqsize / (ps_bins - 1)
    pcenter = -o["PhaseSpaceShiftY"] * pqsize / (ps_bins - 1)
    p.update(ps_bins=ps_bins, pqsize=pqsize,
             qmin=qcenter - pqsize / 2, qmax=qcenter + pqsize / 2,
             pmin=pcenter - pqsize / 2, pmax=pcenter + pqsize / 2)
    sE, E0 = o["BeamEnergySpread"], o["BeamEnergy"]
    dE = sE * E0
    f_rev = float(o["RevolutionFrequency"])
    R_bend = (o["BendingRadius"] if o["BendingRadius"] > 0
              else C / (2 * math.pi * f_rev))
    H = float(o["HarmonicNumber"])
    f_RF = f_rev * H
    gamma = E0 / ME_EV
    V0 = E_CHARGE * gamma ** 4 / (3 * EPS0 * R_bend)
    V_RF = o["AcceleratingVoltage"]
    V_eff = math.sqrt(V_RF * V_RF - V0 * V0)
    fs, alpha0 = o["SyncFreq"], o["alpha0"]
    if fs == 0:
        fs = f_rev * math.sqrt(alpha0 * H * V_eff / (2 * math.pi * E0))
    else:
        alpha0 = (math.copysign(1, fs) * 2 * math.pi * E0 / (H * V_eff)
                  * (fs / f_rev) ** 2)
    alpha = [alpha0, o["alpha1"], o["alpha2"]]
    bl = C * dE / H / f_rev ** 2 / V_eff * fs
    if o["StepsPerRevolution"] > 0:
        steps = o["StepsPerRevolution"] * f_rev / fs
    else:
        steps = max(int(o["StepsPerTs"]), 1)
    calc_damp = E0 / V0 / f_rev     # E0*e/W0/f_rev with W0 = V0*e
    t_damp = calc_damp if o["DampingTime"] < 0 else o["DampingTime"]
    dt = 1.0 / (fs * steps)
    revolutionpart = f_rev * dt
    angle = 2 * math.pi / steps
    bunchspacing = 1.0 / f_RF
    spacing_ps = bunchspacing * C / bl / pqsize
    spacing_bins = int(round(ps_bins * spacing_ps))
    fmax = ps_bins * C / (pqsize * bl)
    padding = max(o["padding"], 1.0)
    padded_bins = int(math.ceil(ps_bins * padding))
    if o["RoundPadding"]:
        padded_bins = upper_power_of_two(padded_bins)
    e1 = 2.0 / (fs * t_damp * steps) if t_damp > 0 else 0.0
    slip = [angle, alpha[1] / alpha[0] * angle, alpha[2] / alpha[0] * angle]
    I_norm = (I_ALFVEN / ME_EV * 2 * math.pi * (dE * fs / f_rev) ** 2
              / V_eff / H * (bl / R_bend) ** (1.0 / 3.0))
    currents = list(o["BunchCurrent"])
    if "S_csr" in kw:
        currents = [kw["S_csr"] * I_norm]
    Ib = sum(c for c in currents if c > 0)
    dp = pqsize / (ps_bins - 1)
    p.update(
        sE=sE, E0=E0, dE=dE, f_rev=f_rev, R_bend=R_bend, H=H, f_RF=f_RF,
        V0=V0, V_RF=V_RF, V_eff=V_eff, fs=fs, alpha=alpha, bl=bl,
        steps=steps, t_damp=t_damp, dt=dt, revolutionpart=revolutionpart,
        angle=angle, spacing_bins=spacing_bins, fmax=fmax,
        padded_bins=padded_bins, e1=e1, slip=slip, I_norm=I_norm, Ib=Ib,
        S_csr=Ib / I_norm, gap=o["VacuumGap"], fc=o["CutoffFreq"],
        laststep=int(math.ceil(steps * o["rotations"])),
        # wake scaling of the ElectricField (inc/PS/ElectricField.hpp:99)
        wakescaling=Ib * dt * C / bl / (dp * sE * E0),
        # RFKickMap bl2phase (src/SM/RFKickMap.cpp:29)
        bl2phase=bl / C * f_RF * 2 * math.pi,
        axes=(qcenter - pqsize / 2, qcenter + pqsize / 2, bl,
              pcenter - pqsize / 2, pcenter + pqsize / 2, dE),
    )
    return p


def wakescaling_for(p, Ib):
    """ElectricField wake scaling for another bunch current."""
    dp = p["pqsize"] / (p["ps_bins"] - 1)
    return Ib * p["dt"] * C / p["bl"] / (dp * p["sE"] * p["E0"])


def fill_desc(desc, p, chain, Ib=None, impedance=0, it=None, clamp=False):
    """Fill a BunchDesc (of the C ABI or of the oracle) for one bunch.

    chain 0 is the solver loop of src/main.cpp:948-1053 (linear or
    sinusoidal RF kick, drift, Fokker-Planck, wake kick); chain 1 is the
    rotation scheme (RotationMap, wake kick, Fokker-Planck)."""
    o = p["opts"]
    desc.n = p["ps_bins"]
    desc.chain = chain
    desc.it = int(o["InterpolationPoints"] if it is None else it)
    desc.clamp = int(clamp)
    axes = p["axes"]
    if hasattr(desc, "axes"):
        for k in range(6):
            desc.axes[k] = axes[k]
    else:
        (desc.qmin, desc.qmax, desc.qscale, desc.pmin, desc.pmax,
         desc.pscale) = axes
    desc.zoom = o["InitialDistZoom"]
    desc.angle = p["angle"]
    desc.rf_linear = int(bool(o["LinearRF"]))
    desc.rf_angle = p["angle"]
    desc.rf_revpart = p["revolutionpart"]
    desc.rf_vrf = p["V_eff"]
    desc.rf_v0 = p["V0"]
    desc.rf_bl2phase = p["bl2phase"]
    desc.rf_phase = math.asin(p["V0"] / p["V_eff"])
    for k in range(3):
        desc.slip[k] = p["slip"][k]
    desc.nslip = 3
    desc.e0 = p["E0"]
    desc.e1 = p["e1"]
    desc.fptype = int(o["FPType"])
    desc.derivation = int(o["derivation"])
    ib = p["Ib"] if Ib is None else Ib
    desc.wakescaling = wakescaling_for(p, ib)
    desc.renormalize = int(o["RenormalizeCharge"])
    if hasattr(desc, "impedance"):
        desc.impedance = impedance
    return desc


def wake_impedance_args(p):
    """Arguments of makeImpedance for the wake (single bucket)."""
    o = p["opts"]
    return dict(nfreqs=p["padded_bins"], fmax=p["fmax"], R_bend=p["R_bend"],
                frev=p["f_rev"], gap=p["gap"], use_csr=bool(o["UseCSR"]),
                s=o["WallConductivity"], xi=o["WallSusceptibility"],
                inner_coll_radius=o["CollimatorRadius"])


def csr_impedance_args(p):
    """makeImpedance for the radiated CSR (src/main.cpp:723-727)."""
    return dict(nfreqs=p["padded_bins"], fmax=p["fmax"], R_bend=p["R_bend"],
                frev=p["f_rev"], gap=p["gap"] if p["gap"] > 0 else -1.0)


def run_file(p, chain=0, it=None, clamp=False, steps=1, csr=False, Ib=None,
             warmup=0):
    """The "key = value" run file of the C++ solver driver
    (inovesa_gb300/cpp/vfps_solver.cpp) for derived parameters p: `warmup`
    untimed steps, then `steps` timed ones."""
    o = p["opts"]
    a = p["axes"]
    w = wake_impedance_args(p)
    c = csr_impedance_args(p)
    slip = [float(v) for v in p["slip"]]
    kv = dict(
        n=p["ps_bins"], chain=chain,
        it=int(o["InterpolationPoints"] if it is None else it),
        clamp=int(bool(clamp)), renormalize=int(o["RenormalizeCharge"]),
        qmin=a[0], qmax=a[1], qscale=a[2], pmin=a[3], pmax=a[4], pscale=a[5],
        Ib=p["Ib"] if Ib is None else Ib, f_rev=p["f_rev"],
        zoom=o["InitialDistZoom"], padded_bins=w["nfreqs"], fmax=w["fmax"],
        R_bend=w["R_bend"], gap=w["gap"], use_csr=int(w["use_csr"]),
        s=w["s"], xi=w["xi"], coll=w["inner_coll_radius"],
        csr_gap=c["gap"], spacing_bins=p["spacing_bins"],
        revolutionpart=p["revolutionpart"], E0=p["E0"], sE=p["sE"],
        dt=p["dt"], linear_rf=int(bool(o["LinearRF"])), angle=p["angle"],
        f_RF=p["f_RF"], V_eff=p["V_eff"], V0=p["V0"], nslip=len(slip),
        e1=p["e1"], fptype=int(o["FPType"]), fptrack=int(o["FPTrack"]),
        derivation=int(o["derivation"]), fc=p["fc"], csr=int(bool(csr)),
        steps=int(steps), warmup=int(warmup))
    for k, v in enumerate(slip):
        kv["slip%d" % k] = v
    return "".join("%s = %r\n" % (k, float(v)) for k, v in kv.items())
