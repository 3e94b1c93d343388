"""Extract golden vectors from the reference's unit tests into JSON.

Run once where the Inovesa sources are available, with the path of the
source tree (the directory that holds test/) as the only argument:

    python tests/golden/make_golden.py <inovesa source tree>

It reads the Boost.Test sources under test/ as text (nothing is compiled or
run) and writes tests/golden/reference_tests.json with, per test case, the
mesh set-up, the input data and the expected values that the reference
asserts.  The parity tests then run the same cases through the oracle and
the CUDA path.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _cases(text):
    """Yield (name, body) for every BOOST_*TEST_CASE* in a source file."""
    pat = re.compile(r"BOOST_(?:AUTO|FIXTURE)_TEST_CASE(?:_TEMPLATE)?\s*\(\s*"
                     r"(\w+)[^)]*\)\s*\{")
    for m in pat.finditer(text):
        depth, i = 1, m.end()
        while depth and i < len(text):
            depth += {"{": 1, "}": -1}.get(text[i], 0)
            i += 1
        yield m.group(1), text[m.end():i - 1]


def _num_list(s):
    return [float(v.rstrip("f")) for v in
            re.findall(r"-?\d+(?:\.\d*)?(?:e-?\d+)?f?", s)]


def _vectors(body):
    """std::vector<...> name{{ ... }} initialisers -> {name: [numbers]}."""
    out = {}
    for m in re.finditer(r"std::vector<[^>]*>\s+(\w+)\s*\{\{(.*?)\}\};", body,
                         re.S):
        out[m.group(1)] = _num_list(m.group(2))
    return out


def _positions(body, name):
    m = re.search(r"std::vector<vfps::PhaseSpace::Position>\s+" + name
                  + r"\s*\{(.*?)\};", body, re.S)
    if not m:
        return None
    pairs = re.findall(r"\{\s*([-\d.ef]+)\s*,\s*([-\d.ef]+)\s*\}", m.group(1))
    return [[float(a.rstrip("f")), float(b.rstrip("f"))] for a, b in pairs]


def _balanced_args(body, start):
    """Text between the parenthesis at body[start] and its partner."""
    depth, i = 0, start
    while i < len(body):
        depth += {"(": 1, ")": -1}.get(body[i], 0)
        if depth == 0:
            return body[start + 1:i]
        i += 1
    return body[start + 1:]


def _ps_axes(body):
    m = re.search(r"make_shared<vfps::PhaseSpace>\(([^;]*?)nullptr", body,
                  re.S)
    vals = _num_list(m.group(1))
    return vals[:6]


_ANGLES = {"half_pi": 1.5707963267948966, "pi": 3.141592653589793}
_ITYPES = {"none": 1, "linear": 2, "quadratic": 3, "cubic": 4}


def rotation_cases(text):
    out = []
    for name, body in _cases(text):
        vec = _vectors(body)
        m = re.search(r"vfps::RotationMap\s*(?:rm)?\s*\(", body)
        if not m:
            continue
        args = _balanced_args(body, m.end() - 1)
        angle = re.search(r"constants::(\w+)<", args).group(1)
        itype = re.search(r"InterpolationType::(\w+)", args).group(1)
        after = args.split("InterpolationType::" + itype, 1)[1]
        toks = [t.strip() for t in after.split(",") if t.strip()]
        clamp = toks[0] == "true"
        rotmap = toks[1]
        n = 4
        rotmapsize = n * n if "size()" in rotmap else int(rotmap)
        case = dict(name=name, n=n, axes=_ps_axes(body),
                    angle=_ANGLES[angle], it=_ITYPES[itype], clamp=clamp,
                    rotmapsize=rotmapsize,
                    throws="BOOST_CHECK_THROW" in body,
                    data_in=vec.get("data1"), data_out=vec.get("data2"))
        pm = re.search(r"Position p1\{([^}]*)\}.*?Position p2\{([^}]*)\}",
                       body, re.S)
        if pm:
            case["particle_in"] = _num_list(pm.group(1))
            case["particle_out"] = _num_list(pm.group(2))
        tol = re.search(r"BOOST_CHECK_SMALL\(ps2->getData\(\)\[i\]-data2\[i\],"
                        r"\s*static_cast<vfps::meshdata_t>\(([\d.e-]+)\)", body)
        case["tolerance"] = float(tol.group(1)) if tol else None
        out.append(case)
    return out


def kick_cases(text):
    out = []
    for name, body in _cases(text):
        vec = _vectors(body)
        itype = re.search(r"InterpolationType::(\w+)", body).group(1)
        axis = re.search(r"KickMap::Axis::(\w)", body).group(1)
        pos_in = []
        pm = re.search(r"for\(uint32_t i=0; i<(\d+); i\+\+\)\{\s*pos\.push_back"
                       r"\(\{([\d.f]+)\*i,([\d.f]+)\*i\}\);", body)
        if pm:
            cnt, fx, fy = int(pm.group(1)), float(pm.group(2).rstrip("f")), \
                float(pm.group(3).rstrip("f"))
            pos_in = [[fx * i, fy * i] for i in range(cnt)]
        out.append(dict(name=name, n=4, axes=_ps_axes(body),
                        it=_ITYPES[itype], axis=0 if axis == "x" else 1,
                        offset=vec["offset"], data_in=vec["data1"],
                        data_out=vec["data2"], pos_in=pos_in,
                        pos_out=_positions(body, "pos2"), tolerance=1e-5))
    return out


def phasespace_cases(text):
    out = {}
    for name, body in _cases(text):
        m = re.search(r"resetSize\((\d+)\s*,\s*(\w+(?:\.size\(\))?)\)", body)
        vec = _vectors(body)
        entry = dict(n=int(m.group(1)) if m else None)
        pm = re.search(r"vfps::PhaseSpace\s+ps1\(([^;]*?)\);", body, re.S)
        if pm is None:
            pm = re.search(r"vfps::PhaseSpace\(([^;]*?)\),\s*std::", body,
                           re.S)
        if pm:
            entry["axes"] = _num_list(pm.group(1).split("nullptr")[0])[:6]
        if "buckets" in vec:
            entry["buckets"] = vec["buckets"]
        if "data1" in vec:
            entry["data1"] = vec["data1"]
        if "data2" in vec:
            entry["data2"] = vec["data2"]
        entry["throws"] = "BOOST_CHECK_THROW" in body
        closes = re.findall(r"BOOST_CHECK_CLOSE\(([^;]*)\);", body)
        entry["checks_close"] = [c.strip() for c in closes]
        smalls = re.findall(r"BOOST_CHECK_SMALL\(([^;]*)\);", body)
        entry["checks_small"] = [c.strip() for c in smalls]
        out[name] = entry
    return out


def electric_field_fixture(text):
    fx = {}
    m = re.search(r"bunchspacing\s*=\s*([\d.]+)", text)
    fx["bunchspacing"] = float(m.group(1))
    m = re.search(r"uint32_t n\s*=\s*(\d+)", text)
    fx["n"] = int(m.group(1))
    m = re.search(r"ConstImpedance>\(spaced_bins,\s*([\de.]+)", text)
    fx["z_fmax"] = float(m.group(1))
    m = re.search(r"make_shared<vfps::PhaseSpace>\(\s*([^;]*?)nullptr", text,
                  re.S)
    fx["axes"] = _num_list(m.group(1))[:6]
    m = re.search(r"make_shared<vfps::ElectricField>\(\s*ps, z, buckets, "
                  r"spacing_bins, nullptr,\s*([^;]*?)\);", text, re.S)
    vals = _num_list(m.group(1))
    fx["f_rev"], fx["revolutionpart"], fx["Ib"], fx["E0"], \
        fx["sigma_delta"], fx["dt"] = vals[:6]
    fx["fillings"] = [_num_list(f) for f in
                      re.findall(r"filling\(\{([^}]*)\}\)", text)]
    m = re.search(r"FreeSpaceCSR\(eff\.spaced_bins,\s*([\de.]+),\s*([\de.]+)",
                  text)
    fx["fs_csr_frev"], fx["fs_csr_fmax"] = float(m.group(1)), \
        float(m.group(2))
    for key, pat in (("change_magnitude", r"change_magnitude\s*=\s*([\de.-]+)"),
                     ("change_epsilon", r"change_epsilon\s*=\s*([\de.-]+)"),
                     ("change_limit", r"change_limit\s*=\s*([\de.-]+)")):
        fx[key] = float(re.search(pat, text).group(1))
    m = re.search(r"wake_potential\[b\]\[x\]\s*-padded_profile\[b\]\[x\]\*"
                  r"scaling,\s*static_cast<vfps::integral_t>\(([\de.-]+)\)",
                  text)
    fx["wake_z1_tolerance"] = float(m.group(1))
    m = re.search(r"BOOST_CHECK_CLOSE\(correct_solution\[x\], "
                  r"test_solution\[x\], ([\de.-]+)\)", text)
    fx["padding_tolerance_percent"] = float(m.group(1))
    return fx


def ruler_case(text):
    m = re.search(r"Ruler<int32_t> axis1\((\d+),(-?\d+),(-?\d+)", text)
    z = re.search(r"axis1\.zerobin\(\),\s*(\d+)", text)
    return dict(steps=int(m.group(1)), min=float(m.group(2)),
                max=float(m.group(3)), zerobin=float(z.group(1)))


def impedance_cases(ref):
    with open(os.path.join(ref, "test", "impedance.dat")) as f:
        rows = [list(map(float, line.split())) for line in f if line.strip()]
    with open(os.path.join(ref, "test", "TestConstImpedance.cpp")) as f:
        t = f.read()
    n = int(re.search(r"size_t n = (\d+)", t).group(1))
    z = float(re.search(r"impedance_t Z = ([\de.]+)", t).group(1))
    return dict(impedance_dat=rows, const_n=n, const_z=z)


def main(ref):
    def rd(name):
        with open(os.path.join(ref, "test", name)) as f:
            return f.read()
    out = dict(
        source="Inovesa test/ sources, parsed by tests/golden/make_golden.py",
        rotation=rotation_cases(rd("TestRotationMap.cpp")),
        kick=kick_cases(rd("TestKickMap.cpp")),
        phasespace=phasespace_cases(rd("TestPhaseSpace.cpp")),
        electric_field=electric_field_fixture(rd("TestElectricField.cpp")),
        ruler=ruler_case(rd("TestRuler.cpp")),
        impedance=impedance_cases(ref),
    )
    path = os.path.join(HERE, "reference_tests.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <inovesa source tree>")
    main(sys.argv[1])
