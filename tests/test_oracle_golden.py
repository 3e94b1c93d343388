"""The oracle against the reference's own golden vectors (CPU only).

Each test restates one reference unit test with the numbers extracted into
tests/golden/reference_tests.json; both the float restatement (the
reference CPU stand-in) and the FP64 oracle must pass it.
"""
import math

import numpy as np
import pytest

import oracle
from tests.refcases import ef_fixture, gauss_projection

DTYPES = [np.float32, np.float64]


@pytest.mark.parametrize("dtype", DTYPES)
def test_rotation_golden(golden, dtype):
    """test/TestRotationMap.cpp:18-205."""
    for case in golden["rotation"]:
        n = case["n"]
        args = (case["axes"], case["angle"], case["it"], case["clamp"],
                case["rotmapsize"])
        if case["throws"]:
            with pytest.raises(ValueError):
                oracle.rotation(np.zeros((n, n)), *args[:4],
                                rotmapsize=args[4], dtype=dtype)
            continue
        data = np.array(case["data_in"]).reshape(n, n)
        out = oracle.rotation(data, case["axes"], case["angle"], case["it"],
                              case["clamp"], rotmapsize=case["rotmapsize"],
                              dtype=dtype)[0]
        np.testing.assert_allclose(out.ravel(), case["data_out"], rtol=0,
                                   atol=case["tolerance"], err_msg=case["name"])
        if "particle_in" in case:
            p = oracle.rotation_particle(n, case["axes"], case["angle"],
                                         case["particle_in"], dtype=dtype)
            np.testing.assert_allclose(p, case["particle_out"], atol=1e-3)


@pytest.mark.parametrize("dtype", DTYPES)
def test_kick_golden(golden, dtype):
    """test/TestKickMap.cpp:18-172 (maps and particles)."""
    for case in golden["kick"]:
        n = case["n"]
        data = np.array(case["data_in"]).reshape(n, n)
        out = oracle.kick(case["axis"], data, case["it"], case["offset"],
                          dtype=dtype)[0]
        np.testing.assert_allclose(out.ravel(), case["data_out"], rtol=0,
                                   atol=case["tolerance"], err_msg=case["name"])
        for pin, pout in zip(case["pos_in"], case["pos_out"]):
            p = oracle.kick_particle(case["axis"], n, case["offset"], pin,
                                     dtype=dtype)
            np.testing.assert_allclose(p, pout, atol=case["tolerance"],
                                       err_msg=case["name"])


def test_ruler_golden(golden):
    """test/TestRuler.cpp:13-26."""
    r = golden["ruler"]
    for dtype in DTYPES:
        _, _, zb = oracle.ruler(r["steps"], r["min"], r["max"], dtype)
        assert zb == r["zerobin"]


@pytest.mark.parametrize("dtype", DTYPES)
def test_phasespace_golden(golden, dtype):
    """test/TestPhaseSpace.cpp:38-132."""
    ps = golden["phasespace"]
    c = ps["one_bucket"]
    r = oracle.ps_init(c["n"], c["axes"], dtype=dtype)
    assert abs(r["integral"] - 1) <= 1e-3
    _, delta, _ = oracle.ruler(c["n"], c["axes"][0], c["axes"][1], dtype)
    assert abs(delta / (24 / (32 - 1.0)) - 1) <= 1e-3
    # copy constructor keeps the integral
    r2 = oracle.ps_init(c["n"], c["axes"], data=r["data"], dtype=dtype)
    assert abs(r2["integral"] - 1) <= 1e-3

    c = ps["two_buckets"]
    r = oracle.ps_init(c["n"], c["axes"], filling=c["buckets"], dtype=dtype)
    assert abs(r["integral"] - 1) <= 1e-3
    np.testing.assert_allclose(r["filling"], c["buckets"], rtol=1e-3)

    c = ps["five_buckets"]
    fs = np.array(c["buckets"])
    r = oracle.ps_init(c["n"], c["axes"], filling=fs, dtype=dtype)
    assert abs(r["integral"] - 1) <= 1e-3
    nz = fs > 0
    np.testing.assert_allclose(r["filling"][nz], fs[nz], rtol=1e-3)
    assert np.all(r["filling"][~nz] == 0)
    qa, dq, _ = oracle.ruler(c["n"], c["axes"][0], c["axes"][1], dtype)
    pa, dp, _ = oracle.ruler(c["n"], c["axes"][3], c["axes"][4], dtype)
    mq, vq = oracle.moments(qa, dq, r["projx"], fs, r["filling"], dtype)
    mp, vp = oracle.moments(pa, dp, r["projy"], fs, r["filling"], dtype)
    assert np.all(np.abs(mq) <= 1e-3) and np.all(np.abs(mp) <= 1e-3)
    np.testing.assert_allclose(np.sqrt(vq[nz]), 1, rtol=1e-3)
    np.testing.assert_allclose(np.sqrt(vp[nz]), 1, rtol=1e-3)
    assert np.all(vq[~nz] == 0) and np.all(vp[~nz] == 0)

    c = ps["no_norm"]
    with pytest.raises(ValueError):
        oracle.ps_init(c["n"], c["axes"], filling=c["buckets"], dtype=dtype)

    c = ps["datacopy"]
    r = oracle.ps_init(c["n"], c["axes"], filling=c["buckets"],
                       data=np.array(c["data1"]).reshape(2, c["n"], c["n"]),
                       dtype=dtype)
    np.testing.assert_array_equal(r["data"].ravel(),
                                  np.array(c["data1"], dtype))


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("pattern_index", [0, 1])
def test_electric_field_golden(golden, dtype, pattern_index):
    """test/TestElectricField.cpp:98-239: padding layout, Z=1 wake equals
    the scaled profile, and free-space CSR only acts forward."""
    fx = golden["electric_field"]
    pattern = fx["fillings"][pattern_index]
    e = ef_fixture(fx, pattern)
    n = e["n"]
    r = oracle.ps_init(n, e["axes"], filling=e["bunches"], dtype=dtype)
    proj = r["projx"]
    zc = oracle.z_const(e["nmax"], 1.0)
    wake = oracle.wake_potential(proj, zc, e["wakescaling"], e["buckets"],
                                 e["spacing"], dtype=dtype)
    # padding: bunch b sits at bucket_b * spacing (pattern walked reversed)
    qa, _, _ = oracle.ruler(n, e["axes"][0], e["axes"][1], dtype)
    qa = qa.astype(np.float64)
    expect = np.zeros(e["nmax"])
    for bucket, norm in enumerate(reversed(pattern)):
        expect[bucket * e["spacing"]:bucket * e["spacing"] + n] = \
            norm * gauss_projection(qa)
    got = np.zeros(e["nmax"])
    for b, bk in enumerate(e["buckets"]):
        got[bk * e["spacing"]:bk * e["spacing"] + n] = proj[b]
    nzm = expect != 0
    rel = np.abs(got[nzm] - expect[nzm]) / np.abs(expect[nzm])
    assert rel.max() <= fx["padding_tolerance_percent"] / 100 * 2
    # Z = 1: wake potential equals profile * scaling
    scaling = np.float32(np.float32(e["wakescaling"]) / np.float32(e["nmax"]))
    assert np.max(np.abs(wake - proj * scaling)) <= fx["wake_z1_tolerance"]
    # forward wake of free-space CSR
    z0 = oracle.z_const(e["nmax"], 0.0)
    zfs = oracle.z_free_space(e["nmax"], fx["fs_csr_frev"], fx["fs_csr_fmax"])
    z = (z0 + zfs).astype(np.complex64)
    w0 = oracle.wake_potential(proj, z, e["wakescaling"], e["buckets"],
                               e["spacing"], dtype=dtype)
    mod = proj.copy()
    cf = n // 2
    for b in range(mod.shape[0]):
        d = fx["change_magnitude"] * mod[b, cf]
        mod[b, cf] -= d
        mod[b, cf + 1] += d
        mod[b, cf + 2] += d
        mod[b, cf + 3] -= d
    w1 = oracle.wake_potential(mod, z, e["wakescaling"], e["buckets"],
                               e["spacing"], dtype=dtype)
    change = np.abs(w0 - w1)
    for b in range(mod.shape[0]):
        assert change[b].max() >= fx["change_limit"]
        assert change[b, :cf].max() <= fx["change_limit"]


def test_const_impedance_golden(golden):
    """test/TestConstImpedance.cpp:15-27."""
    g = golden["impedance"]
    z = oracle.z_const(g["const_n"], g["const_z"])
    expect = np.zeros(g["const_n"], np.complex64)
    expect[:g["const_n"] // 2] = g["const_z"]
    np.testing.assert_array_equal(z, expect)


def test_airy_against_scipy():
    """Own Airy functions (ParallelPlatesCSR input) against scipy."""
    special = pytest.importorskip("scipy.special")
    for x in np.concatenate([np.linspace(0, 3, 61), np.linspace(3, 104, 203)]):
        (ai, aip, bi, bip), ovf = oracle.airy(x)
        A, Ap, B, Bp = special.airy(x)
        assert not ovf
        for got, ref in ((ai, A), (aip, Ap), (bi, B), (bip, Bp)):
            if np.isfinite(ref):
                assert abs(got - ref) <= 1e-11 * abs(ref) + 1e-300, \
                    (x, got, ref)
    (_, _, bi, bip), ovf = oracle.airy(120.0)
    assert ovf


def test_rfft_against_numpy():
    rng = np.random.default_rng(1)
    for n in (8, 512, 768):
        x = rng.standard_normal(n)
        got = oracle.rfft(x)[: n // 2 + 1]
        np.testing.assert_allclose(got, np.fft.rfft(x), rtol=0, atol=1e-9)
