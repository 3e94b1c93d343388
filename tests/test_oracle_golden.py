"""The oracle against the reference's own golden vectors (CPU only).

Each test restates one reference unit test with the numbers extracted into
tests/golden/reference_tests.json; both the float restatement (the
reference CPU stand-in) and the FP64 oracle must pass it.  The units the
reference has no test for (ParallelPlatesCSR, ResistiveWall, the
Fokker-Planck stencils, the Drift and RF offsets) are checked against a
second, independent statement in numpy and scipy.
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


def parallel_plates_scipy(nfreqs, f0, f_max, g):
    """ParallelPlatesCSR::__calcImpedance (src/Z/ParallelPlatesCSR.cpp:
    25-70) evaluated independently of the oracle: numpy and scipy's
    exponentially scaled Airy functions (airye: Ai e^z, Bi e^-z with
    z = 2/3 u^1.5), FP64.  Each term is formed from the scaled values (the
    exponentials cancel in Ai Bi), and the sum over odd p ends at the
    first p whose Bi or Bi' exceeds the largest double, where the
    reference's Boost call throws; cast to complex64 as the reference
    stores it."""
    special = pytest.importorskip("scipy.special")
    c = 2.99792458e8
    z0 = 1.0 / (8.854187817e-12 * c)          # inc/defines.hpp:48-54
    f0 = float(np.float32(f0))
    f_max = float(np.float32(f_max))
    delta = f_max / f0 / (nfreqs - 1.0)
    r_bend = c / (2 * np.pi * f0)
    out = np.zeros(nfreqs, np.complex64)
    for i in range(1, nfreqs // 2 + 1):
        n = i * delta
        m = n * (g / r_bend) ** 1.5
        maxp = int(2 * m * (r_bend / g) ** 1.5 * f0 * g / c)
        b = m ** (-4.0 / 3.0)
        p = np.arange(1, maxp + 1, 2, dtype=np.float64)
        u = np.pi ** 2 * p * p / 2 ** (2.0 / 3.0) * b
        eai, eaip, ebi, ebip = special.airye(u)
        zeta = 2.0 / 3.0 * u ** 1.5
        big = np.log(np.finfo(np.float64).max)
        with np.errstate(divide="ignore"):
            over = (np.log(np.abs(ebi)) + zeta > big) \
                | (np.log(np.abs(ebip)) + zeta > big)
        if over.any():
            k = int(np.argmax(over))
            eai, eaip, ebi, ebip = eai[:k], eaip[:k], ebi[:k], ebip[:k]
            u, zeta = u[:k], zeta[:k]
        ai, aip = eai * np.exp(-zeta), eaip * np.exp(-zeta)
        z = np.sum(aip * aip - 1j * eaip * ebip
                   + u * (ai * ai - 1j * eai * ebi))
        z *= 4.0 * b * n * g / r_bend * np.pi ** 2 * 2 ** (1.0 / 3.0) * z0
        out[i] = np.complex64(z)
    return out


def test_parallel_plates_against_scipy():
    """The oracle's ParallelPlatesCSR table (the reference has no test of
    it) against the independent evaluation above, for the benchmark's
    lattice (g/R = 0.006) and a wider gap: within FP32 rounding of each
    entry (2e-6 relative) plus 1e-6 of the largest."""
    for nfreqs, f0, f_max, g in ((512, 9.0e6, 3.173436465819893e12,
                                  0.03180896772824628),
                                 (1024, 2.7e6, 4.0e11, 0.05)):
        want = parallel_plates_scipy(nfreqs, f0, f_max, g)
        got = oracle.z_parallel_plates(nfreqs, f0, f_max, g)
        scale = np.abs(want).max()
        assert scale > 0
        np.testing.assert_allclose(got, want, rtol=2e-6, atol=1e-6 * scale)


def test_resistive_wall_restated():
    """The oracle's ResistiveWall table (src/Z/ResistiveWall.cpp:24-57; no
    reference test) against a numpy statement of the same float
    arithmetic: bit for bit."""
    c = 2.99792458e8
    z0 = 376.730313461                         # inc/Z/Impedance.hpp:94
    for n, f0, f_max, L, s, xi, b in ((512, 9.0e6, 3.17e12, 33.3, 5.8e7,
                                       0.0, 0.0159),
                                      (2048, 2.7e6, 4.0e11, 10.0, 1.4e6,
                                       0.1, 0.02)):
        f0_32, fmax_32 = np.float32(f0), np.float32(f_max)
        z1r = np.float32(np.sqrt(z0 * (1 + xi) * float(f0_32) / s / np.pi
                                 / c) * L / 2 / b)
        delta = np.float32(float(fmax_32 / f0_32) / (n - 1.0))
        want = np.zeros(n, np.complex64)
        for i in range(n // 2 + 1):
            r = np.sqrt(np.float32(i) * delta)
            want[i] = np.complex64(complex(z1r * r, -(z1r * r)))
        got = oracle.z_resistive_wall(n, f0, f_max, L, s, xi, b)
        np.testing.assert_array_equal(got, want)


def fp_stencils_numpy(n, pmin, pmax, e1, fptype, derivation):
    """FokkerPlanckMap's stencil table (src/SM/FokkerPlanckMap.cpp:30-118;
    no reference test) stated in numpy, FP64, with the reference's
    operation order; the energy axis from the oracle's Ruler (itself pinned
    to test/TestRuler.cpp)."""
    pv, dp, zb = oracle.ruler(n, pmin, pmax)
    e1_2d = e1 / (2.0 * dp)
    e1_6d = e1 / (6.0 * dp)
    e1_d2 = e1 / (dp * dp)
    damp = fptype in (1, 3)
    diff = fptype in (2, 3)
    ip = derivation
    idx = np.zeros((n, ip), np.uint32)
    w = np.zeros((n, ip))
    if derivation == 3:
        for j in range(1, n - 1):
            pos = pv[j]
            idx[j] = (j - 1, j, j + 1)
            w[j] = (0.0, 1.0, 0.0)
            if damp:
                w[j, 0] += -e1_2d * pos
                w[j, 1] += e1
                w[j, 2] += e1_2d * pos
            if diff:
                w[j, 0] += e1_d2
                w[j, 1] += -2.0 * e1_d2
                w[j, 2] += e1_d2
    else:
        j = 2
        while j < zb:
            pos = pv[j]
            idx[j] = (j - 2, j - 1, j, j + 1)
            w[j] = (0.0, 0.0, 1.0, 0.0)
            if damp:
                w[j, 0] += e1_6d * 1.0 * pos
                w[j, 1] += e1_6d * -6.0 * pos
                w[j, 2] += e1 + e1_6d * 3.0 * pos
                w[j, 3] += e1_6d * 2.0 * pos
            if diff:
                w[j, 1] += e1_d2
                w[j, 2] += -2.0 * e1_d2
                w[j, 3] += e1_d2
            j += 1
        # the second loop starts at the truncated centre (an integer index
        # initialised from the axis' zero bin): on a mesh whose centre lies
        # between two columns it rewrites the last one of the first loop
        j = int(zb)
        while j < n - 2:
            pos = pv[j]
            idx[j] = (j - 1, j, j + 1, j + 2)
            w[j] = (0.0, 1.0, 0.0, 0.0)
            if damp:
                w[j, 0] += e1_6d * -2.0 * pos
                w[j, 1] += e1 + e1_6d * -3.0 * pos
                w[j, 2] += e1_6d * 6.0 * pos
                w[j, 3] += e1_6d * -1.0 * pos
            if diff:
                w[j, 0] += e1_d2
                w[j, 1] += -2.0 * e1_d2
                w[j, 2] += e1_d2
            j += 1
    return idx.ravel(), w.ravel()


@pytest.mark.parametrize("derivation", [3, 4])
@pytest.mark.parametrize("fptype", [0, 1, 2, 3])
@pytest.mark.parametrize("n", [64, 255, 256])
def test_fp_stencils_restated(n, fptype, derivation):
    """The oracle's Fokker-Planck stencils against the numpy statement
    above: the same indices, weights equal to FP64 rounding."""
    axes = (-6.0, 6.0, 2e-3, -6.0, 6.0, 6.11e5)
    e1 = 2.0 / (100 * 500) * 50
    idx, w = oracle.fp_stencils(n, axes, e1, fptype, derivation)
    idx_n, w_n = fp_stencils_numpy(n, axes[3], axes[4], e1, fptype,
                                   derivation)
    np.testing.assert_array_equal(idx, idx_n)
    np.testing.assert_allclose(w, w_n, rtol=1e-14, atol=1e-16)


def test_drift_and_rf_offsets_restated():
    """The oracle's DriftMap offsets (src/SM/DriftMap.cpp:21-30) and static
    RFKickMap offsets (src/SM/RFKickMap.cpp:59-83, linear and sinusoidal;
    no reference test of either) against numpy statements of the same
    formulas, FP64, on axes from the oracle's Ruler."""
    n = 200
    axes = (-6.0, 6.0, 1.7e-3, -5.0, 7.0, 4.3e5)
    qv, dq, zq = oracle.ruler(n, axes[0], axes[1])
    pv, dp, zp = oracle.ruler(n, axes[3], axes[4])
    slip = [2.1e-3, 3.0e-4, -5.0e-5]
    e0 = 1.3e9
    want = np.zeros(n)
    for i, s in enumerate(slip):
        want += s * pv * (pv * axes[5] / e0) ** i
    want /= dq
    got = oracle.drift_offsets(n, axes, slip, e0)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-300)
    angle, bl2phase = 0.0125, 0.37
    want = np.tan(angle) * (zq - np.arange(n)) \
        + np.tan(angle) * 0.0 / bl2phase / dq
    got = oracle.rf_offsets(n, axes, True, angle=angle, bl2phase=bl2phase)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13)
    revpart, vrf, v0, phase = 0.5, 1.1e6, 9.0e4, 0.3
    want = revpart * (-1.0 * vrf * np.sin(qv * bl2phase + phase) + v0) \
        / dp / axes[5]
    got = oracle.rf_offsets(n, axes, False, revpart=revpart, vrf=vrf, v0=v0,
                            bl2phase=bl2phase, phase=phase)
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-13)
