"""The reference's own unit tests, run through the CUDA path.

Same cases and tolerances as test/TestRotationMap.cpp, test/TestKickMap.cpp,
test/TestPhaseSpace.cpp, test/TestElectricField.cpp,
test/TestImpedance.cpp and test/TestConstImpedance.cpp (numbers from
tests/golden/reference_tests.json).
"""
import os

import numpy as np
import pytest

from inovesa_gb300 import vfps as V
from tests.refcases import ef_fixture, gauss_projection

pytestmark = pytest.mark.gpu


def _ps(ctx, axes, n, filling=(1.0,), data=None, zoom=1.0):
    return V.PhaseSpace(*axes, ctx, 1, 1, filling, zoom, data, n=n)


def test_rotation_maps(gpu_ctx, golden):
    for c in golden["rotation"]:
        n = c["n"]
        d1 = np.array(c["data_in"] or np.zeros(n * n)).reshape(1, n, n)
        ps1 = _ps(gpu_ctx, c["axes"], n, data=d1)
        ps2 = _ps(gpu_ctx, c["axes"], n)
        if c["throws"]:
            with pytest.raises(V.InvalidArgument):
                V.RotationMap(ps1, ps2, n, n, c["angle"], c["it"], c["clamp"],
                              c["rotmapsize"])
            continue
        rm = V.RotationMap(ps1, ps2, n, n, c["angle"], c["it"], c["clamp"],
                           c["rotmapsize"])
        rm.apply()
        np.testing.assert_allclose(ps2.getData().ravel(), c["data_out"],
                                   rtol=0, atol=c["tolerance"],
                                   err_msg=c["name"])
        if "particle_in" in c:
            p = rm.applyTo(np.array(c["particle_in"], np.float32))
            np.testing.assert_allclose(p.ravel(), c["particle_out"], atol=1e-3)


def test_kick_maps(gpu_ctx, golden):
    for c in golden["kick"]:
        n = c["n"]
        ps1 = _ps(gpu_ctx, c["axes"], n,
                  data=np.array(c["data_in"]).reshape(1, n, n))
        ps2 = _ps(gpu_ctx, c["axes"], n)
        km = V.KickMap(ps1, ps2, c["it"], False, c["axis"])
        km.swapOffset(c["offset"])
        km.apply()
        pos = km.applyToAll(np.array(c["pos_in"], np.float32))
        np.testing.assert_allclose(pos, c["pos_out"], atol=c["tolerance"],
                                   err_msg=c["name"])
        np.testing.assert_allclose(ps2.getData().ravel(), c["data_out"],
                                   rtol=0, atol=c["tolerance"],
                                   err_msg=c["name"])


def test_phasespace(gpu_ctx, golden):
    g = golden["phasespace"]
    c = g["one_bucket"]
    ps1 = _ps(gpu_ctx, c["axes"], c["n"])
    assert abs(ps1.getIntegral() - 1) <= 1e-3
    ps2 = ps1.copy()
    assert abs(ps2.getIntegral() - 1) <= 1e-3
    assert abs(ps2.getDelta(0) / (24 / (32 - 1.0)) - 1) <= 1e-3
    assert abs(ps2.getDelta(1) / (24 / (32 - 1.0)) - 1) <= 1e-3

    c = g["two_buckets"]
    ps = _ps(gpu_ctx, c["axes"], c["n"], filling=c["buckets"])
    assert abs(ps.getIntegral() - 1) <= 1e-3
    np.testing.assert_allclose(ps.getBunchPopulation(), c["buckets"],
                               rtol=1e-3)

    c = g["five_buckets"]
    fs = np.array(c["buckets"])
    ps = _ps(gpu_ctx, c["axes"], c["n"], filling=fs)
    assert abs(ps.getIntegral() - 1) <= 1e-3
    pop = ps.getBunchPopulation()
    nz = fs > 0
    np.testing.assert_allclose(pop[nz], fs[nz], rtol=1e-3)
    ps.variance(0)
    ps.variance(1)
    assert np.all(np.abs(ps.getMoment(0, 0)) <= 1e-3)
    assert np.all(np.abs(ps.getMoment(1, 0)) <= 1e-3)
    np.testing.assert_allclose(ps.getBunchLength()[nz], 1, rtol=1e-3)
    np.testing.assert_allclose(ps.getEnergySpread()[nz], 1, rtol=1e-3)
    assert np.all(ps.getBunchLength()[~nz] == 0)
    assert np.all(ps.getEnergySpread()[~nz] == 0)

    c = g["no_norm"]
    with pytest.raises(V.InvalidArgument):
        _ps(gpu_ctx, c["axes"], c["n"], filling=c["buckets"])

    c = g["datacopy"]
    d1 = np.array(c["data1"], np.float32)
    ps = _ps(gpu_ctx, c["axes"], c["n"], filling=c["buckets"], data=d1)
    np.testing.assert_array_equal(ps.getData().ravel(), d1)

    c = g["swap"]
    d2 = np.array(c["data2"], np.float32)
    ps1 = _ps(gpu_ctx, c["axes"], c["n"], filling=c["buckets"], data=d1)
    ps2 = _ps(gpu_ctx, c["axes"], c["n"], filling=c["buckets"], data=d2)
    ps1.swap(ps2)
    np.testing.assert_array_equal(ps2.getData().ravel(), d1)
    np.testing.assert_array_equal(ps1.getData().ravel(), d2)
    ps1.swap(ps2)
    np.testing.assert_array_equal(ps1.getData().ravel(), d1)

    c = g["assign"]
    ps1 = _ps(gpu_ctx, c["axes"], c["n"], filling=c["buckets"], data=d1)
    ps2 = _ps(gpu_ctx, c["axes"], c["n"], filling=c["buckets"], data=d2)
    ps2.assign(ps1)
    np.testing.assert_array_equal(ps1.getData().ravel(), d1)
    np.testing.assert_array_equal(ps2.getData().ravel(), d1)

    c = g["projection_setter"]
    ps = _ps(gpu_ctx, c["axes"], c["n"])
    xs = np.arange(c["n"], dtype=np.float32) + 0.5
    ps.setProjection(0, 0, xs)
    np.testing.assert_allclose(ps.getProjection(0, 0), xs, rtol=1e-3)


@pytest.mark.parametrize("pattern_index", [0, 1])
def test_electric_field(gpu_ctx, golden, pattern_index):
    fx = golden["electric_field"]
    pattern = fx["fillings"][pattern_index]
    e = ef_fixture(fx, pattern)
    n = e["n"]
    ps = _ps(gpu_ctx, e["axes"], n, filling=e["bunches"])
    z = V.ConstImpedance(gpu_ctx, e["nmax"], fx["z_fmax"], 1)
    f = V.ElectricField.wake(ps, z, e["buckets"], e["spacing"], gpu_ctx,
                             fx["f_rev"], fx["revolutionpart"], fx["Ib"],
                             fx["E0"], fx["sigma_delta"], fx["dt"])
    assert list(f._ps.getBunchPopulation() > 0) == [True] * len(e["bunches"])
    # padding layout
    f.padBunchProfiles()
    qa = ps.getAxis(0).astype(np.float64)
    expect = np.zeros(e["nmax"])
    for bucket, norm in enumerate(reversed(pattern)):
        expect[bucket * e["spacing"]:bucket * e["spacing"] + n] = \
            norm * gauss_projection(qa)
    got = f.getPaddedBunchProfiles()
    nzm = expect != 0
    assert np.all(got[~nzm] == 0)
    rel = np.abs(got[nzm] - expect[nzm]) / expect[nzm]
    assert rel.max() <= fx["padding_tolerance_percent"] / 100 * 2
    # Z = 1: wake equals profile * scaling
    wake = f.wakePotential()
    proj = ps.getProjection(0)
    assert np.max(np.abs(wake - proj * f.getWakeScaling())) \
        <= fx["wake_z1_tolerance"]
    # free-space CSR acts forward only
    z0 = V.ConstImpedance(gpu_ctx, e["nmax"], fx["z_fmax"], 0)
    z0 += V.FreeSpaceCSR(gpu_ctx, e["nmax"], fx["fs_csr_frev"],
                         fx["fs_csr_fmax"])
    f2 = V.ElectricField.wake(ps, z0, e["buckets"], e["spacing"], gpu_ctx,
                              fx["f_rev"], fx["revolutionpart"], fx["Ib"],
                              fx["E0"], fx["sigma_delta"], fx["dt"])
    w0 = f2.wakePotential()
    mod = proj.copy()
    cf = n // 2
    for b in range(mod.shape[0]):
        d = fx["change_magnitude"] * mod[b, cf]
        mod[b, cf] -= d
        mod[b, cf + 1] += d
        mod[b, cf + 2] += d
        mod[b, cf + 3] -= d
        ps.setProjection(0, b, mod[b])
    w1 = f2.wakePotential()
    change = np.abs(w0 - w1)
    for b in range(mod.shape[0]):
        assert change[b].max() >= fx["change_limit"]
        assert change[b, :cf].max() <= fx["change_limit"]


def test_impedances(gpu_ctx, golden, tmp_path):
    g = golden["impedance"]
    z = V.ConstImpedance(gpu_ctx, g["const_n"], 1e9, g["const_z"])
    expect = np.zeros(g["const_n"], np.complex64)
    expect[:g["const_n"] // 2] = g["const_z"]
    np.testing.assert_array_equal(z.data(), expect)
    # file read-in (test/impedance.dat)
    path = os.path.join(tmp_path, "impedance.dat")
    with open(path, "w") as fh:
        for row in g["impedance_dat"]:
            fh.write("%d\t%g\t%g\n" % (int(row[0]), row[1], row[2]))
    zf = V.Impedance.from_file(gpu_ctx, path, 1e9)
    assert zf.nFreqs() == len(g["impedance_dat"])
    np.testing.assert_array_equal(
        zf.data(), np.array([complex(r[1], r[2]) for r in g["impedance_dat"]],
                            np.complex64))
    # constructors, addition, swap (test/TestImpedance.cpp:15-86)
    zv = np.zeros(8, np.complex64)
    zv[5] = 0.5j
    z1 = V.Impedance(gpu_ctx, zv, 1e9)
    assert z1[0] == 0 and z1[5] == 0.5j
    assert abs(z1.fmax() - 1e9) <= 1e-3 * 1e9
    z2 = z1.copy()
    assert z2[5] == 0.5j
    i8 = np.arange(8)
    zv1 = (i8 + 1j * (-i8 + 4)).astype(np.complex64)
    zv2 = ((i8 - 2) + 3j).astype(np.complex64)
    a = V.Impedance(gpu_ctx, zv1, 1e9)
    b = V.Impedance(gpu_ctx, zv2, 1e9)
    c = a + b
    np.testing.assert_array_equal(c.data(), zv1 + zv2)
    a += b
    np.testing.assert_array_equal(b.data(), zv2)
    np.testing.assert_array_equal(a.data(), c.data())
    d = a.copy()
    a.swap(b)
    np.testing.assert_array_equal(a.data(), zv2)
    np.testing.assert_array_equal(b.data(), c.data())
    np.testing.assert_array_equal(d.data(), b.data())
