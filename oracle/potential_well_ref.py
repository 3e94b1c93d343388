"""Test infrastructure only: the CPU restatement (FP64 numpy) of the
potential-well start that vfps_batch_potential_well computes on the
device.  Only tests/ and the warm-start experiment's checks use it.

The reference names this start as an option it ignores
(HaissinskiIterations, src/IO/ProgramOptions.cpp:270, "currently
ignored"), so there is no reference code to follow; the restatement is the
published physics, built on the reference's own per-step quantities:

* the RF kick offsets of every row (src/SM/RFKickMap.cpp:59-78) and the
  drift offsets of every column (src/SM/DriftMap.cpp:21-30), both through
  this oracle's C restatement (oracle_rf_offsets, oracle_drift_offsets);
* the wake kick offsets of a profile (src/PS/ElectricField.cpp wake
  potential, oracle_wake_potential).

A kick map with offset o moves the density by -o, so the y-kick of row x
is F(x) = -(rf(x) + wake(x)) and the drift moves a cell by -d(y).  The
continuous-time invariant of the step is Phi(x) + G(y) (Phi, G the
integrals of F and d: the Haissinski potential well); the split step
(kick, then drift) conserves Phi + G + F d / 2 to first order (the
Baker-Campbell-Hausdorff term of the two maps).  The Fokker-Planck term
holds the energy spread at one unit, which fixes the scale T = slip0 /
(dq dp).  The density is exp(-E / T), the profile enters the wake, and
the profile iterates to a fixed point.

The rotation chain (chain 1) rotates the mesh exactly, which conserves the
radial invariant; its state takes the rotation's quadratic potential and
kinetic term as a linear kick and drift of the same angle, and only the
wake kick enters the split-step term (with the sign of a kick after the
rotation, the better of the two signs under the restated rotation step).
"""
import numpy as np

import oracle


def _simpson(n, d):
    w = np.full(n, 2.0)
    w[1::2] = 4.0
    w[0] = w[-1] = 1.0
    return w * d / 3.0


def _trapezoid(f):
    out = np.zeros_like(f)
    out[1:] = np.cumsum(0.5 * (f[1:] + f[:-1]))
    return out


def offsets(p, chain=0):
    """(rf offsets per row, drift offsets per column, dq, dp, T) of the
    step of derived parameters p (inovesa_gb300.params.derive).  Chain 0:
    the RF kick and the drift of the kick-drift step.  Chain 1 (the
    rotation by `angle` per step, src/SM/RotationMap.cpp): the linear kick
    and drift of the same angle (the rotation's quadratic potential and
    kinetic term, in mesh cells, both axes in units of the spreads)."""
    n, axes, o = p["ps_bins"], p["axes"], p["opts"]
    _, dq, zq = oracle.ruler(n, axes[0], axes[1])
    pv, dp, _ = oracle.ruler(n, axes[3], axes[4])
    if chain == 1:
        th = p["angle"]
        rf = np.tan(th) * (zq - np.arange(n))
        dr = th * pv / dq
        return rf, dr, dq, dp, th / (dq * dp)
    rf = oracle.rf_offsets(n, axes, bool(o["LinearRF"]), angle=p["angle"],
                           revpart=p["revolutionpart"], vrf=p["V_eff"],
                           v0=p["V0"], bl2phase=p["bl2phase"],
                           phase=np.arcsin(p["V0"] / p["V_eff"]))
    dr = oracle.drift_offsets(n, axes, p["slip"], p["E0"])
    T = p["slip"][0] / (dq * dp)
    return rf, dr, dq, dp, T


def _cross(F, wake, chain):
    """Half the row factor of the split-step term E += f(x) d(y): the whole
    y-kick after the kick-drift step (chain 0); for the rotation chain only
    the wake kick, with the sign of a kick that follows the rotation (the
    rotation itself conserves the radial invariant exactly)."""
    return 0.5 * F if chain == 0 else 0.5 * wake


def state(p, Z, wakescaling, iterations=200, mix=0.5, fill=1.0, chain=0):
    """(density [x][y], last relative L1 change of the profile) of the
    potential-well start; Z the wake impedance (None: no wake)."""
    n = p["ps_bins"]
    rf, dr, dq, dp, T = offsets(p, chain)
    wsx, wsy = _simpson(n, dq), _simpson(n, dp)
    G = _trapezoid(dr)
    G -= G.min()
    rho = np.zeros(n)
    last = iterations if Z is not None else 0
    change = 0.0
    for it in range(last + 1):
        wake = (oracle.wake_potential(rho, Z, wakescaling)[0]
                if Z is not None and it > 0 else np.zeros(n))
        F = -(rf + wake)
        Phi = _trapezoid(F)
        e = -(Phi[:, None] + G[None, :]
              + _cross(F, wake, chain)[:, None] * dr[None, :]) / T
        psi = np.exp(e - e.max())
        psi *= fill / np.einsum("xy,x,y->", psi, wsx, wsy)
        if it == last:
            return psi, change
        new = psi @ wsy
        change = (np.abs(new - rho).sum() / np.abs(rho).sum()
                  if it > 0 else 1.0)
        rho = new if it == 0 else rho + mix * (new - rho)
    raise AssertionError("unreachable")


def beam_states(p, Z, wakescaling, buckets, spacing, fills, iterations=200,
                mix=0.5):
    """(densities [member][x][y], last relative L1 changes) of the
    potential-well start of a multi-bunch beam: the members share the
    derived parameters p and one padded profile (their buckets `spacing`
    mesh cells apart, src/PS/ElectricField.cpp:255-263), so each member's
    wake carries the fields of all members' profiles of the previous
    iteration; member m is normalised to fills[m]."""
    n = p["ps_bins"]
    nb = len(fills)
    rf, dr, dq, dp, T = offsets(p)
    wsx, wsy = _simpson(n, dq), _simpson(n, dp)
    G = _trapezoid(dr)
    G -= G.min()
    rho = np.zeros((nb, n))
    change = np.zeros(nb)
    last = iterations if Z is not None else 0
    for it in range(last + 1):
        wake = (oracle.wake_potential(rho, Z, wakescaling, buckets=buckets,
                                      spacing=spacing)
                if Z is not None and it > 0 else np.zeros((nb, n)))
        out = []
        for m in range(nb):
            F = -(rf + wake[m])
            Phi = _trapezoid(F)
            e = -(Phi[:, None] + G[None, :]
                  + 0.5 * F[:, None] * dr[None, :]) / T
            psi = np.exp(e - e.max())
            psi *= fills[m] / np.einsum("xy,x,y->", psi, wsx, wsy)
            out.append(psi)
        if it == last:
            return out, change
        new = np.stack([psi @ wsy for psi in out])
        if it > 0:
            change = (np.abs(new - rho).sum(axis=1)
                      / np.abs(rho).sum(axis=1))
        else:
            change = np.ones(nb)
        rho = new if it == 0 else rho + mix * (new - rho)
    raise AssertionError("unreachable")
