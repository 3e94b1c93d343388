// One bunch through the reference's solver loop, written against the C++
// façade (include/vfps.hpp) the way src/main.cpp is written against the
// reference classes: set-up as in src/main.cpp:469-760, steps as in
// src/main.cpp:948-1053 (chain 0: wake kick, RF kick, drift,
// Fokker-Planck; chain 1: rotation, wake kick, Fokker-Planck).
//
// The derived parameters (src/main.cpp:163-355, inovesa_gb300/params.py)
// come as "key = value" lines in a run file, so the program is only the
// solver loop.  Usage:
//     vfps_solver RUNFILE OUTPREFIX
// writes OUTPREFIX.density (nx*nx float32 after the last step),
// OUTPREFIX.profile (nx float32), OUTPREFIX.csr (the CSR power of every
// step, one per line, when csr = 1) and OUTPREFIX.timing ("steps seconds"
// of the timed steps: the run file's optional "warmup" steps run first,
// untimed; the device is synchronised before the clock starts and before
// it stops).  Exit status 0 on success; errors are printed and give status
// 1.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "vfps.hpp"

namespace {

std::map<std::string, double> read_run_file(const char* path)
{
    std::ifstream in(path);
    if (!in) {
        throw std::runtime_error(std::string("cannot open ") + path);
    }
    std::map<std::string, double> p;
    std::string line;
    while (std::getline(in, line)) {
        const auto eq = line.find('=');
        if (line.empty() || line[0] == '#' || eq == std::string::npos) {
            continue;
        }
        std::string k = line.substr(0, eq), v = line.substr(eq + 1);
        k.erase(0, k.find_first_not_of(" \t"));
        k.erase(k.find_last_not_of(" \t") + 1);
        p[k] = std::stod(v);
    }
    return p;
}

double get(const std::map<std::string, double>& p, const char* k)
{
    const auto it = p.find(k);
    if (it == p.end()) {
        throw std::invalid_argument(std::string("run file lacks ") + k);
    }
    return it->second;
}

void write_floats(const std::string& path, const std::vector<float>& v)
{
    std::ofstream out(path, std::ios::binary);
    out.write(reinterpret_cast<const char*>(v.data()),
              std::streamsize(v.size() * sizeof(float)));
}

int run(const char* runfile, const std::string& prefix)
{
    using namespace vfps;
    const auto p = read_run_file(runfile);
    const uint32_t n = uint32_t(get(p, "n"));
    const int chain = int(get(p, "chain"));
    const int it = int(get(p, "it"));
    const bool clamp = get(p, "clamp") != 0;
    const int renormalize = int(get(p, "renormalize"));
    const double f_rev = get(p, "f_rev"), Ib = get(p, "Ib");
    const double revolutionpart = get(p, "revolutionpart");

    auto ctx = std::make_shared<Context>(0);
    // PhaseSpace (src/main.cpp:469-525): the Gaussian start
    auto t1 = std::make_shared<PhaseSpace>(
        get(p, "qmin"), get(p, "qmax"), get(p, "qscale"), get(p, "pmin"),
        get(p, "pmax"), get(p, "pscale"), ctx, Ib / f_rev, Ib,
        std::vector<float>{1.f}, get(p, "zoom"), n);
    if (renormalize >= 0) {
        t1->updateXProjection();
        t1->normalize();
    }
    auto t2 = std::make_shared<PhaseSpace>(*t1);
    auto t3 = std::make_shared<PhaseSpace>(*t1);

    // wake impedance and field (src/main.cpp:717-755)
    auto zw = makeImpedance(ctx, size_t(get(p, "padded_bins")),
                            float(get(p, "fmax")), get(p, "R_bend"), f_rev,
                            get(p, "gap"), get(p, "use_csr") != 0,
                            get(p, "s"), get(p, "xi"), get(p, "coll"));
    std::unique_ptr<ElectricField> field;
    if (zw) {
        field.reset(new ElectricField(
            t1, zw, {0u}, uint32_t(get(p, "spacing_bins")), ctx, f_rev,
            revolutionpart, Ib, get(p, "E0"), get(p, "sE"), get(p, "dt")));
    }
    // the radiated CSR (src/main.cpp:723-727)
    const bool csr = get(p, "csr") != 0;
    std::unique_ptr<ElectricField> rdtn;
    if (csr) {
        auto zr = makeImpedance(ctx, size_t(get(p, "padded_bins")),
                                float(get(p, "fmax")), get(p, "R_bend"),
                                f_rev, get(p, "csr_gap"));
        rdtn.reset(new ElectricField(t1, zr, {0u}, 0, ctx, f_rev,
                                     revolutionpart));
    }

    // the maps (src/main.cpp:603-716)
    std::unique_ptr<SourceMap> rm, rfm, drm, wm, fpm;
    WakePotentialMap* wkm = nullptr;
    const float angle = float(get(p, "angle"));
    if (chain == 0) {
        if (get(p, "linear_rf") != 0) {
            rfm.reset(new RFKickMap(t2, t1, angle, float(get(p, "f_RF")), it,
                                    clamp, ctx));
        } else {
            rfm.reset(new RFKickMap(t2, t1, float(revolutionpart),
                                    float(get(p, "V_eff")),
                                    float(get(p, "f_RF")),
                                    float(get(p, "V0")), it, clamp, ctx));
        }
        std::vector<float> slip;
        for (int k = 0; k < int(get(p, "nslip")); k++) {
            slip.push_back(float(get(p, ("slip" + std::to_string(k)).c_str())));
        }
        drm.reset(new DriftMap(t1, t3, slip, float(get(p, "E0")), it, clamp,
                               ctx));
        if (field) {
            wkm = new WakePotentialMap(t1, t2, field.get(), it, clamp, ctx);
            wm.reset(wkm);
        } else {
            wm.reset(new Identity(t1, t2, ctx));
        }
    } else {
        rm.reset(new RotationMap(t1, t2, n, n, angle, it, clamp,
                                 clamp ? size_t(n) * n : 0, ctx));
        if (field) {
            wkm = new WakePotentialMap(t2, t3, field.get(), it, clamp, ctx);
            wm.reset(wkm);
        } else {
            wm.reset(new Identity(t2, t3, ctx));
        }
    }
    const float e1 = float(get(p, "e1"));
    if (e1 > 0) {
        fpm.reset(new FokkerPlanckMap(t3, t1, n, n, int(get(p, "fptype")),
                                      int(get(p, "fptrack")), e1,
                                      int(get(p, "derivation")), ctx));
    } else {
        fpm.reset(new Identity(t3, t1, ctx));
    }

    // the solver loop (src/main.cpp:948-1053)
    const long steps = long(get(p, "steps"));
    const auto wu = p.find("warmup");
    const long warmup = wu == p.end() ? 0 : long(wu->second);
    const float fc = float(get(p, "fc"));
    std::vector<float> csr_power;
    auto t0 = std::chrono::steady_clock::now();
    for (long s = 0; s < warmup + steps; s++) {
        if (s == warmup) {
            ctx->synchronize();
            t0 = std::chrono::steady_clock::now();
        }
        if (wkm) {
            wkm->update();
        }
        if (renormalize > 0 && s % renormalize == 0) {
            t1->integrateAndNormalize();
        } else {
            t1->integrate();
        }
        if (rdtn) {
            csr_power.push_back(rdtn->updateCSR(fc)[0]);
        }
        if (chain == 0) {
            wm->apply();
            rfm->apply();
            drm->apply();
            fpm->apply();
        } else {
            rm->apply();
            wm->apply();
            fpm->apply();
        }
        t1->updateXProjection();
    }
    ctx->synchronize();
    const double seconds = std::chrono::duration<double>(
        std::chrono::steady_clock::now() - t0).count();
    {
        std::ofstream out(prefix + ".timing");
        out.precision(9);
        out << steps << " " << seconds << "\n";
    }
    write_floats(prefix + ".density", t1->getData());
    write_floats(prefix + ".profile", t1->getProjection(0));
    if (rdtn) {
        std::ofstream out(prefix + ".csr");
        out.precision(9);
        for (float v : csr_power) {
            out << v << "\n";
        }
    }
    if (ctx->deviceStatus() != 0) {
        throw std::runtime_error("device error status after the run");
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 3) {
        std::cerr << "usage: vfps_solver RUNFILE OUTPREFIX\n";
        return 2;
    }
    try {
        return run(argv[1], argv[2]);
    } catch (const std::exception& e) {
        std::cerr << "vfps_solver: " << e.what() << "\n";
        return 1;
    }
}
