"""CUDA path against the oracle, one operation at a time, on realistic
meshes (64^2 .. 256^2).  Tolerances: single maps within 2e-6 (relative
to the largest density) of the float restatement and 1e-5 relative L1 of
the FP64 oracle; FP64-built tables within 1e-5 relative."""
import math

import numpy as np
import pytest

import oracle
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V

pytestmark = pytest.mark.gpu

AXES = (-6.0, 6.0, 2e-3, -6.0, 6.0, 6.11e5)


def rel_l1(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).sum()
                 / np.abs(np.asarray(b, np.float64)).sum())


def density(n, seed=0, skew=0.3):
    """A smooth, asymmetric, positive test density."""
    rng = np.random.default_rng(seed)
    q = np.linspace(-6, 6, n)
    g = np.exp(-0.5 * (q[:, None] ** 2 + (q[None, :] - skew) ** 2))
    g *= 1 + 0.2 * np.sin(q[:, None] + 0.7 * q[None, :])
    g += 1e-3 * rng.random((n, n))
    return (g / g.sum()).astype(np.float32)[None]


def _ps(ctx, n, data=None, axes=AXES):
    return V.PhaseSpace(*axes, ctx, 1, 1, [1.0], 1.0, data, n=n)


@pytest.mark.parametrize("n", [64, 256])
@pytest.mark.parametrize("it,clamp", [(2, False), (3, False), (4, False),
                                      (4, True)])
def test_rotation(gpu_ctx, n, it, clamp):
    d = density(n, seed=n + it)
    angle = 2 * math.pi / 500 * 7
    a = _ps(gpu_ctx, n, d)
    b = _ps(gpu_ctx, n)
    V.RotationMap(a, b, n, n, angle, it, clamp, n * n if clamp else 0).apply()
    got = b.getData()
    ref32 = oracle.rotation(d, AXES, angle, it, clamp, dtype=np.float32)
    ref64 = oracle.rotation(d, AXES, angle, it, clamp, dtype=np.float64)
    assert np.max(np.abs(got - ref32)) <= 2e-6 * np.abs(ref32).max()
    assert rel_l1(got, ref64) <= 1e-5


@pytest.mark.parametrize("axis", [0, 1])
@pytest.mark.parametrize("it", [2, 3, 4])
def test_kick(gpu_ctx, axis, it):
    n = 128
    rng = np.random.default_rng(axis * 10 + it)
    d = density(n, seed=it)
    count = n  # one bunch: n offsets either way
    off = rng.uniform(-3.5, 3.5, count).astype(np.float32)
    off[:3] = [-n, n / 2 + 0.25, -(n / 2) - 0.5]   # far out of the mesh
    a = _ps(gpu_ctx, n, d)
    b = _ps(gpu_ctx, n)
    km = V.KickMap(a, b, it, False, axis)
    km.swapOffset(off)
    km.apply()
    got = b.getData()
    np.testing.assert_array_equal(km.getForce(), off)
    ref32 = oracle.kick(axis, d, it, off, dtype=np.float32)
    ref64 = oracle.kick(axis, d, it, off, dtype=np.float64)
    assert np.max(np.abs(got - ref32)) <= 2e-6 * np.abs(ref32).max()
    assert rel_l1(got, ref64) <= 1e-5


def test_static_kick_offsets(gpu_ctx):
    """DriftMap and RFKickMap offsets (src/SM/DriftMap.cpp:21-30,
    src/SM/RFKickMap.cpp:59-83) against the oracle."""
    p = P.derive(GridSize=128, StepsPerTs=500, alpha1=1e-3, alpha2=2e-4)
    n = 128
    a, b = _ps(gpu_ctx, n, axes=p["axes"]), _ps(gpu_ctx, n, axes=p["axes"])
    dm = V.DriftMap(a, b, p["slip"], p["E0"], 4, False)
    ref = oracle.drift_offsets(n, p["axes"], p["slip"], p["E0"],
                               dtype=np.float32)
    np.testing.assert_allclose(dm.getForce(), ref, rtol=2e-6, atol=1e-9)
    rf = V.RFKickMap(b, a, p["angle"], p["f_RF"], 4, False)
    ref = oracle.rf_offsets(n, p["axes"], True, angle=p["angle"],
                            bl2phase=p["bl2phase"], dtype=np.float32)
    np.testing.assert_allclose(rf.getForce(), ref, rtol=2e-6, atol=1e-9)
    rfs = V.RFKickMap.sinusoidal(b, a, p["revolutionpart"], p["V_eff"],
                                 p["f_RF"], p["V0"], 4, False)
    ref = oracle.rf_offsets(n, p["axes"], False, revpart=p["revolutionpart"],
                            vrf=p["V_eff"], v0=p["V0"],
                            bl2phase=p["bl2phase"],
                            phase=math.asin(p["V0"] / p["V_eff"]),
                            dtype=np.float64)
    np.testing.assert_allclose(rfs.getForce(), ref, rtol=1e-4,
                               atol=1e-6 * np.abs(ref).max())


@pytest.mark.parametrize("derivation", [3, 4])
@pytest.mark.parametrize("fptype", [0, 1, 2, 3])
def test_fokker_planck(gpu_ctx, derivation, fptype):
    n = 128
    d = density(n, seed=derivation + fptype)
    e1 = 2.0 / (100 * 500) * 50   # a strong decrement to expose errors
    a, b = _ps(gpu_ctx, n, d), _ps(gpu_ctx, n)
    V.FokkerPlanckMap(a, b, n, n, fptype, 0, e1, derivation).apply()
    got = b.getData()
    for dt, tol in ((np.float32, None), (np.float64, 1e-5)):
        idx, w = oracle.fp_stencils(n, AXES, e1, fptype, derivation, dtype=dt)
        ref = oracle.fp_apply(d, derivation, idx, w, dtype=dt)
        if tol is None:
            assert np.max(np.abs(got - ref)) <= 2e-6 * np.abs(ref).max()
        else:
            assert rel_l1(got, ref) <= tol


def test_identity(gpu_ctx):
    d = density(32)
    a, b = _ps(gpu_ctx, 32, d), _ps(gpu_ctx, 32)
    V.Identity(a, b).apply()
    np.testing.assert_array_equal(b.getData(), d)


def test_projections_and_normalize(gpu_ctx):
    n = 256
    d = np.concatenate([density(n, 1), 2 * density(n, 2)])
    ps = V.PhaseSpace(*AXES, gpu_ctx, 1, 1, [0.5, 0.5], 1.0, d, n=n)
    ws = oracle.simpson(n, AXES[0], AXES[1], np.float64)
    px = oracle.project_x(d, ws)
    py = oracle.project_y(d, ws)
    np.testing.assert_allclose(ps.getProjection(0), px, rtol=2e-6,
                               atol=1e-7 * px.max())
    ps.updateYProjection()
    np.testing.assert_allclose(ps.getProjection(1), py, rtol=2e-6,
                               atol=1e-7 * py.max())
    fill, tot = oracle.integrate(px, ws)
    np.testing.assert_allclose(ps.getBunchPopulation(), fill, rtol=2e-6)
    assert abs(ps.getIntegral() - tot) <= 2e-6 * tot
    ps.normalize()
    ref = oracle.normalize(d, [0.5, 0.5], fill)
    assert rel_l1(ps.getData(), ref) <= 1e-6
    ps.variance(0)
    qa = ps.getAxis(0)
    avg, var = oracle.moments(qa, ps.getDelta(0), px, [0.5, 0.5], fill)
    np.testing.assert_allclose(ps.getMoment(0, 0), avg, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(ps.getMoment(0, 1), var, rtol=1e-5)


def test_gaussian_start(gpu_ctx):
    n = 128
    ps = V.PhaseSpace(*AXES, gpu_ctx, 1, 1, [1.0], 1.3, None, n=n)
    ref = oracle.ps_init(n, AXES, zoom=1.3, dtype=np.float64)
    assert rel_l1(ps.getData(), ref["data"]) <= 1e-6
    assert abs(ps.getIntegral() - ref["integral"]) <= 1e-6


def test_impedance_tables(gpu_ctx):
    p = P.derive(GridSize=256, padding=2.0, VacuumGap=0.0318,
                 WallConductivity=5.8e7)
    n, fmax, f0 = p["padded_bins"], p["fmax"], p["f_rev"]
    fs = V.FreeSpaceCSR(gpu_ctx, n, f0, fmax).data()
    np.testing.assert_allclose(fs, oracle.z_free_space(n, f0, fmax),
                               rtol=1e-6, atol=1e-6 * np.abs(fs).max())
    pp = V.ParallelPlatesCSR(gpu_ctx, n, f0, fmax, 0.0318).data()
    ref = oracle.z_parallel_plates(n, f0, fmax, 0.0318)
    np.testing.assert_allclose(pp, ref, rtol=1e-5,
                               atol=1e-6 * np.abs(ref).max())
    rw = V.ResistiveWall(gpu_ctx, n, f0, fmax, P.C / f0, 5.8e7, 0.0, 0.0159)
    ref = oracle.z_resistive_wall(n, f0, fmax, P.C / f0, 5.8e7, 0.0, 0.0159)
    np.testing.assert_allclose(rw.data(), ref, rtol=1e-6,
                               atol=1e-6 * np.abs(ref).max())
    col = V.CollimatorImpedance(gpu_ctx, n, fmax, 0.0159, 0.005).data()
    np.testing.assert_allclose(col, oracle.z_collimator(n, 0.0159, 0.005),
                               rtol=1e-6)
    args = P.wake_impedance_args(p)
    z = V.makeImpedance(gpu_ctx, **args).data()
    ref = oracle.make_impedance(args["nfreqs"], args["fmax"], args["R_bend"],
                                args["frev"], args["gap"], args["use_csr"],
                                args["s"], args["xi"],
                                args["inner_coll_radius"])
    np.testing.assert_allclose(z, ref, rtol=1e-5,
                               atol=1e-6 * np.abs(ref).max())
    assert V.makeImpedance(gpu_ctx, 64, fmax, p["R_bend"], f0, 0.0) is None


@pytest.mark.parametrize("gap", [-1.0, 0.0318])
def test_wake_and_csr(gpu_ctx, gap):
    p = P.derive(GridSize=256, padding=2.0, VacuumGap=gap, S_csr=0.7)
    n = 256
    d = density(n, seed=5)
    ps = V.PhaseSpace(*p["axes"], gpu_ctx, 1, 1, [1.0], 1.0, d, n=n)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    f = V.ElectricField.wake(ps, z, [0], p["spacing_bins"], gpu_ctx,
                             p["f_rev"], p["revolutionpart"], p["Ib"],
                             p["E0"], p["sE"], p["dt"])
    wake = f.wakePotential()[0]
    proj = ps.getProjection(0)
    ref = oracle.wake_potential(proj, z.data(), float(np.float32(
        p["wakescaling"])))[0]
    assert np.max(np.abs(wake - ref)) <= 1e-5 * np.abs(ref).max()
    # CSR spectrum and power of the same profile
    zr = V.makeImpedance(gpu_ctx, **P.csr_impedance_args(p))
    rd = V.ElectricField(ps, zr, [0], 0, gpu_ctx, p["f_rev"],
                         p["revolutionpart"])
    rd.updateCSR(p["fc"])
    spec = rd.getCSRSpectrum()[0]
    power = rd.getCSRPower()[0]
    rspec, rpower = oracle.csr(proj[0], zr.data(), ps.getDelta(0), p["fc"],
                               P.C / p["bl"])
    assert np.max(np.abs(spec - rspec)) <= 1e-5 * np.abs(rspec).max()
    assert abs(power - rpower) <= 1e-5 * abs(rpower)


def test_multi_bucket_wake(gpu_ctx):
    """Bunches of one beam in buckets 0, 2 and 5 share the padded profile
    (src/PS/ElectricField.cpp:186-263): each bunch's wake carries the
    other bunches' fields at their bucket distance."""
    n, nb = 64, 3
    buckets = [0, 2, 5]
    p = P.derive(GridSize=n, padding=16.0, VacuumGap=0.0318, S_csr=0.5)
    spacing = 3 * n // 2
    rng = np.random.default_rng(9)
    d = rng.random((nb, n, n)).astype(np.float32)
    ps = V.PhaseSpace(*p["axes"], gpu_ctx, 1, 1, [0.5, 0.3, 0.2], 1.0, d,
                      n=n)
    z = V.makeImpedance(gpu_ctx, **P.wake_impedance_args(p))
    f = V.ElectricField.wake(ps, z, buckets, spacing, gpu_ctx, p["f_rev"],
                             p["revolutionpart"], p["Ib"], p["E0"], p["sE"],
                             p["dt"])
    ps.updateXProjection()
    wake = f.wakePotential()
    proj = ps.getProjection(0)
    ref = oracle.wake_potential(proj, z.data(), float(np.float32(
        p["wakescaling"])), buckets=buckets, spacing=spacing)
    assert np.max(np.abs(wake - ref)) <= 1e-5 * np.abs(ref).max()
    # the coupling is there: without the other bunches the wake differs
    alone = oracle.wake_potential(proj[:1], z.data(), float(np.float32(
        p["wakescaling"])))[0]
    assert np.abs(alone - ref[0]).max() > 1e-3 * np.abs(ref[0]).max()
