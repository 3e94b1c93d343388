"""Run output and resume in the layout of the reference's result file.

The reference writes an HDF5 file (src/IO/HDF5File.cpp:45-148) with, per
output step, the bunch population, profile, length and position, the
energy profile, spread and average, the wake potential, the CSR spectrum
and intensity, and every few outputs the phase space; a run can resume
from a saved phase space (src/PS/PhaseSpaceFactory.cpp:19-53).  HDF5 is
not available here, so a run directory holds one NumPy file per dataset,
named after the dataset path ("/BunchProfile/data" ->
BunchProfile.data.npy), with the time axis and the phase-space time axis
alongside.  Datasets are [output step][bunch][...] like the reference's.
"""
import json
import os

import numpy as np

DATASETS = [
    "/Info/AxisValues_z", "/Info/AxisValues_E", "/Info/AxisValues_f",
    "/Info/AxisValues_t", "/Info/BucketNumbers", "/PhaseSpace/axis0",
    "/BunchPopulation/data", "/BunchProfile/data", "/BunchLength/data",
    "/BunchPosition/data", "/EnergyProfile/data", "/EnergySpread/data",
    "/EnergyAverage/data", "/WakePotential/data", "/CSR/Spectrum/data",
    "/CSR/Intensity/data", "/PhaseSpace/data",
]


def _fname(dataset):
    return dataset.strip("/").replace("/", ".") + ".npy"


class Recorder:
    """Collects output steps in memory and writes the run directory on
    flush() / close()."""

    def __init__(self, path, z_axis, e_axis, f_axis=None, buckets=(0,),
                 ps_every=1):
        self.path = path
        os.makedirs(path, exist_ok=True)
        self.ps_every = max(int(ps_every), 1)
        self.static = {
            "/Info/AxisValues_z": np.asarray(z_axis, np.float32),
            "/Info/AxisValues_E": np.asarray(e_axis, np.float32),
            "/Info/BucketNumbers": np.asarray(buckets, np.uint32),
        }
        if f_axis is not None:
            self.static["/Info/AxisValues_f"] = np.asarray(f_axis, np.float64)
        self.series = {}
        self.outputs = 0

    def append(self, t, population, profile, energy_profile, length,
               position, spread, average, wake=None, csr_spectrum=None,
               csr_intensity=None, phase_space=None):
        """One output step (arrays per bunch)."""
        def put(name, v):
            if v is not None:
                self.series.setdefault(name, []).append(np.asarray(v))
        put("/Info/AxisValues_t", np.float64(t))
        put("/BunchPopulation/data", population)
        put("/BunchProfile/data", profile)
        put("/EnergyProfile/data", energy_profile)
        put("/BunchLength/data", length)
        put("/BunchPosition/data", position)
        put("/EnergySpread/data", spread)
        put("/EnergyAverage/data", average)
        put("/WakePotential/data", wake)
        put("/CSR/Spectrum/data", csr_spectrum)
        put("/CSR/Intensity/data", csr_intensity)
        if phase_space is not None and self.outputs % self.ps_every == 0:
            put("/PhaseSpace/data", phase_space)
            put("/PhaseSpace/axis0", np.float64(t))
        self.outputs += 1

    def flush(self):
        for name, v in self.static.items():
            np.save(os.path.join(self.path, _fname(name)), v)
        for name, v in self.series.items():
            np.save(os.path.join(self.path, _fname(name)), np.stack(v))
        with open(os.path.join(self.path, "index.json"), "w") as f:
            json.dump({"datasets": sorted(list(self.static)
                                          + list(self.series)),
                       "outputs": self.outputs}, f)

    close = flush


def read(path, dataset):
    """One dataset of a run directory."""
    return np.load(os.path.join(path, _fname(dataset)))


def resume_state(path, index=-1):
    """(phase space [bunch][x][y], time) of a saved output to restart from
    (the reference's PhaseSpaceFactory from a result file)."""
    ps = read(path, "/PhaseSpace/data")
    t = read(path, "/PhaseSpace/axis0")
    return ps[index], float(t[index])


def record_plain(rec, solver, t, csr=False):
    """Append the state of a PlainSolver (one bunch) to a Recorder."""
    ps = solver.t1
    ps.updateYProjection()
    ps.variance(0)
    ps.variance(1)
    pop = ps.getBunchPopulation()
    prof = ps.getProjection(0)
    eprof = ps.getProjection(1)
    mq, vq, rq = ps._moments(0)
    mp, vp, rp = ps._moments(1)
    wake = (solver.wake_field.getWakePotentials()
            if solver.wake_field is not None else None)
    spec = inten = None
    if csr and solver.rdtn is not None:
        spec = solver.rdtn.getCSRSpectrum()
        inten = solver.rdtn.getCSRPower()
    rec.append(t, pop, prof, eprof, rq, mq, rp, mp, wake, spec, inten,
               ps.getData())
