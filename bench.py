"""Benchmark: phase-space cell-updates/s of the batched current scan.

Workload (one GPU): 256 independent bunches on 256x256 meshes (+-6 sigma),
currents log-spaced over S = 0.01 .. 1.5 (normalised, S = Ib/I_norm),
shared parallel-plates CSR impedance (gap/bend radius 0.006) on a 2x256
padded profile (nmax 512), 1000 steps per synchrotron period, the
reference solver loop (wake kick, RF kick, drift, Fokker-Planck;
src/main.cpp:948-1053).  One bench step = one solver step of all bunches
= one CUDA graph of two kernels (k_bwake: wake potentials, charge
integrals; k_bmaps0: the fused maps and projections).  Synthetic data: the
reference's Gaussian start.

Prints one JSON line (rank 0).  Besides the headline it carries, under
"configs", the other workloads of the benchmark plan measured in the same
run: the plain single bunch on the rotation chain (256x256, 500 steps per
period), the bursting 512x512 bunch with CSR power every step, the uneven
96-bunch batch, the headline scan on the rotation chain and the learned
warm start (periods to equilibrium against the Gaussian start).  --impl
reference times the CPU restatement of the reference solver loop (the
oracle, float) on all host cores on the same workload.
"""
import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("phase-space cell-updates/s on 1 GB300, batched vs plain, "
          "density L1 <=1e-4 vs FP64")
NB, GRID, SPT = 256, 256, 1000
S_MIN, S_MAX = 0.01, 1.5
GAP_OVER_R = 0.006
L2_BYTES = 128 * 2 ** 20     # GB300 L2 (about 126 MiB), rounded up


def workload_params():
    from inovesa_gb300 import params as P
    base = P.derive(GridSize=GRID, StepsPerTs=SPT, padding=2.0)
    gap = GAP_OVER_R * base["R_bend"]
    p = P.derive(GridSize=GRID, StepsPerTs=SPT, padding=2.0, VacuumGap=gap)
    currents = np.geomspace(S_MIN, S_MAX, NB) * p["I_norm"]
    return p, gap, currents


def uneven_workload(seed=4, nb=96, spt=2000):
    """The uneven batch: nb bunches with mesh sides drawn from
    {128, 256, 512, 1024}, currents S ~ U(0.1, 1.5) and interpolation
    orders from {linear, quadratic, cubic} (2..4 points), seeded; the
    parallel-plates gap is 0.006 of the bending radius.  Returns
    [(derived parameters, order)] and the sorted mesh sizes."""
    from inovesa_gb300 import params as P
    rng = np.random.default_rng(seed)
    sizes = rng.choice([128, 256, 512, 1024], size=nb)
    cur = rng.uniform(0.1, 1.5, size=nb)
    its = rng.choice([2, 3, 4], size=nb)
    out = []
    for n, S, it in zip(sizes, cur, its):
        n, it = int(n), int(it)
        p0 = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0)
        p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                     VacuumGap=0.006 * p0["R_bend"], S_csr=float(S))
        out.append((p, it))
    return out, sorted(set(int(v) for v in sizes))


def config_dict(p, gap, l2_note):
    return {
        "workload": "batched current scan: %d bunches x %dx%d FP32, S=%g..%g "
                    "log-spaced, parallel-plates CSR g/R=%g, nmax=%d, "
                    "%d steps/period, reference solver loop (wake kick, RF "
                    "kick, drift, Fokker-Planck)"
                    % (NB, GRID, GRID, S_MIN, S_MAX, GAP_OVER_R,
                       p["padded_bins"], SPT),
        "bunches_per_gpu": NB, "grid": GRID, "nmax": p["padded_bins"],
        "gap_m": gap, "steps_per_period": SPT, "interpolation": "cubic",
        "l2": l2_note,
    }


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_cell():
    """DRAM bytes per cell-update of the step kernel from the committed ncu
    summary, if one exists."""
    path = os.path.join(ROOT, "profiles", "k_bmaps0f_scan256.json")
    try:
        with open(path) as f:
            return float(json.load(f)["dram_bytes_per_cell"])
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,"
         "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"),
                stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [s.strip() for s in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in rows if num(r[2]) is not None]
        pw = [num(r[3]) for r in rows if num(r[3]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].lower().startswith("active")})
        load = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(load) if load else None,
                "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None,
                "samples": len(rows), "reasons": reasons}


def make_batch(ctx, p, currents, z):
    from inovesa_gb300 import params as P
    from inovesa_gb300 import vfps as V
    descs = [P.fill_desc(V.BunchDesc(), p, 0, Ib=float(ib), impedance=0)
             for ib in currents]
    return V.BunchBatch(ctx, descs, [z])


def cpu_baseline(p, currents, z, seconds=12.0):
    """The oracle's float restatement of the reference loop on the host
    cores, on a bounded sample of the workload."""
    import oracle
    from inovesa_gb300 import params as P
    cores = os.cpu_count() or 1
    nb = min(len(currents), max(cores, 1))
    idx = np.linspace(0, len(currents) - 1, nb).astype(int)
    descs = [P.fill_desc(oracle.BunchDesc(), p, 0, Ib=float(currents[i]))
             for i in idx]
    sim = oracle.Sim(descs, Z=z, dtype=np.float32)
    t = time.perf_counter()
    sim.step(2, threads=cores)
    per_step = max((time.perf_counter() - t) / 2, 1e-4)
    steps = max(4, int(seconds / per_step))
    t = time.perf_counter()
    sim.step(steps, threads=cores)
    el = time.perf_counter() - t
    cells = nb * GRID * GRID * steps
    one = oracle.Sim(descs[:1], Z=z, dtype=np.float32)
    s1 = max(4, int(2.0 / (per_step * min(cores, nb) / nb)))
    t = time.perf_counter()
    one.step(s1, threads=1)
    el1 = time.perf_counter() - t
    return {"value": cells / el, "unit": "cell-updates/s", "cores": cores,
            "kind": "port",
            "sample": "%d of the %d bunches, %d solver steps, float "
                      "restatement of the reference loop, %d threads"
                      % (nb, len(currents), steps, cores),
            "single_core_value": GRID * GRID * s1 / el1}


def accuracy_check(batch, start, p, currents, z, threads):
    """Density L1 of the batched FP32 step against the FP64 oracle, from
    the same Gaussian start, for a spread of the scan's bunches: S = 0.01,
    0.1, 0.3, 0.6, 0.9, 1.2, 1.5 (the upper ones above the bursting
    threshold, where FP32 and FP64 trajectories part exponentially, so the
    comparison is made after every one of the first 10 steps and then at
    25, 50 and 100 steps).  The whole 256-bunch batch steps (the
    benchmark's own tiling); returns the worst L1 over the bunches and
    checks, and the per-bunch L1 at 100 steps."""
    import oracle
    from inovesa_gb300 import params as P
    s_norm = np.asarray(currents) / p["I_norm"]
    targets = (0.01, 0.1, 0.3, 0.6, 0.9, 1.2, 1.5)
    idx = [int(np.argmin(np.abs(s_norm - s))) for s in targets]
    descs = [P.fill_desc(oracle.BunchDesc(), p, 0, Ib=float(currents[i]))
             for i in idx]
    ref = oracle.Sim(descs, Z=z, dtype=np.float64)
    batch.upload(start)
    worst, done, last = 0.0, 0, {}
    for check in list(range(1, 11)) + [25, 50, 100]:
        batch.step(check - done)
        ref.step(check - done, threads=threads)
        done = check
        for k, i in enumerate(idx):
            want = ref.density(k)
            got = batch.density(i).astype(np.float64)
            err = float(np.abs(got - want).sum() / np.abs(want).sum())
            worst = max(worst, err)
            last[k] = err
    return {"max_l1": worst, "bar": 1e-4,
            "steps_checked": "1..10, 25, 50, 100 from the Gaussian start",
            "bunches": [{"S": float(s_norm[i]), "l1_at_100": last[k]}
                        for k, i in enumerate(idx)]}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    from inovesa_gb300 import params as P
    import oracle.build
    oracle.build.build()
    p, gap, currents = workload_params()
    z = oracle.make_impedance(p["padded_bins"], p["fmax"], p["R_bend"],
                              p["f_rev"], gap)
    cores = os.cpu_count() or 1
    descs = [P.fill_desc(oracle.BunchDesc(), p, 0, Ib=float(ib))
             for ib in currents]
    sim = oracle.Sim(descs, Z=z, dtype=np.float32)
    sim.step(args.warmup, threads=cores)
    t = time.perf_counter()
    sim.step(args.steps, threads=cores)
    el = time.perf_counter() - t
    cells = NB * GRID * GRID * args.steps
    v = cells / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v,
        "unit": "cell-updates/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": config_dict(p, gap, "host memory"),
        "cpu_baseline": {"value": v, "unit": "cell-updates/s",
                         "cores": cores, "kind": "port",
                         "sample": "the full workload, %d solver steps, "
                                   "float restatement of the reference "
                                   "loop (the reference itself does not "
                                   "build without Boost/FFTW)"
                                   % args.steps},
        "e2e": {"value": v, "unit": "cell-updates/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def rel_l1(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(a - b).sum() / np.abs(b).sum())


def plain_driver(p, chain, it, clamp, steps, warmup, csr=False, Ib=None):
    """The plain one-map-per-launch GPU loop timed inside the C++ driver
    (inovesa_gb300/cpp/vfps_solver.cpp: the reference's main.cpp loop over
    include/vfps.hpp, no interpreter in the loop).  Returns cell-updates/s
    of the timed steps and the density after warmup + steps."""
    from inovesa_gb300 import build as B
    from inovesa_gb300 import params as P
    exe = B.build_driver()
    n = p["ps_bins"]
    with tempfile.TemporaryDirectory() as d:
        rf = os.path.join(d, "run.txt")
        with open(rf, "w") as f:
            f.write(P.run_file(p, chain=chain, it=it, clamp=clamp,
                               steps=steps, csr=csr, warmup=warmup, Ib=Ib))
        out = os.path.join(d, "out")
        r = subprocess.run([exe, rf, out], capture_output=True, text=True,
                           timeout=900)
        if r.returncode != 0:
            raise RuntimeError("vfps_solver failed: " + r.stderr)
        with open(out + ".timing") as f:
            st, sec = f.read().split()
        dens = np.fromfile(out + ".density", np.float32).reshape(n, n)
    return n * n * int(st) / float(sec), dens


def cpu_rate(descs, Z, seconds, threads):
    """The oracle's float restatement of the reference loop on the host
    cores: cell-updates/s over about `seconds`, and the steps sampled."""
    import oracle
    sim = oracle.Sim(descs, Z=Z, dtype=np.float32)
    t = time.perf_counter()
    sim.step(2, threads=threads)
    per = max((time.perf_counter() - t) / 2, 1e-4)
    k = max(2, int(seconds / per))
    t = time.perf_counter()
    sim.step(k, threads=threads)
    cells = sum(int(d.n) ** 2 for d in descs) * k
    return cells / (time.perf_counter() - t), k


def timed_batch(b, stream, steps, warmup):
    """cell-updates/s of back-to-back batched steps (CUDA events on the
    library's stream)."""
    import torch
    b.step(warmup)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(steps)
    e1.record(stream)
    e1.synchronize()
    return b.cells * steps / (e0.elapsed_time(e1) / 1e3)


def config_plain_rotation(ctx, hbm):
    """Plain single bunch: 256x256, cubic RotationMap with clamping, 500
    steps per period, damping time 100 periods, free-space CSR, S = 0.05,
    two synchrotron periods: the plain GPU loop (C++ driver), its density
    against FP64 after the two periods, one host core."""
    import oracle
    from inovesa_gb300 import params as P
    from inovesa_gb300 import vfps as V
    n, spt = 256, 500
    fs = P.derive(GridSize=n, StepsPerTs=spt)["fs"]
    p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=-1.0,
                 S_csr=0.05, DampingTime=100.0 / fs)
    total, warm = 2 * spt, 20
    rate, dens = plain_driver(p, 1, 4, True, total - warm, warm)
    z = V.makeImpedance(ctx, **P.wake_impedance_args(p))
    d = P.fill_desc(oracle.BunchDesc(), p, 1, Ib=p["Ib"], it=4, clamp=True)
    ref = oracle.Sim([d], Z=z.data(), dtype=np.float64)
    ref.step(total)
    cpu1, k1 = cpu_rate([d], z.data(), 3.0, 1)
    return {"workload": "plain single bunch 256x256, cubic RotationMap "
                        "(clamped), 500 steps/period, damping 100 periods, "
                        "free-space CSR, S=0.05, 2 periods",
            "gpu_plain": rate,
            "gpu_plain_driver": "C++ (include/vfps.hpp), one map per launch",
            "density_l1_vs_fp64": rel_l1(dens, ref.density(0)),
            "accuracy_steps": total, "cpu_1core": cpu1,
            "cpu_sample": "%d solver steps, 1 thread" % k1}


def bursting_params(ctx):
    """The bursting bunch: 512x512, 4000 steps per period, S = 1.2,
    parallel-plates CSR (g/R = 0.006) and a resistive wall (5.8e7 S/m):
    its parameters, wake impedance and CSR impedance."""
    from inovesa_gb300 import params as P
    from inovesa_gb300 import vfps as V
    n, spt, S = 512, 4000, 1.2
    p0 = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0)
    p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                 VacuumGap=0.006 * p0["R_bend"], S_csr=S,
                 WallConductivity=5.8e7)
    z = V.makeImpedance(ctx, **P.wake_impedance_args(p))
    zr = V.makeImpedance(ctx, **P.csr_impedance_args(p))
    return p, z, zr


def bursting_batch(ctx, p, z, zr, currents):
    """Bunches of the bursting lattice at the currents given (in units of
    the threshold current's S), each with its CSR power every step."""
    from inovesa_gb300 import params as P
    from inovesa_gb300 import vfps as V
    S = p["S_csr"]
    descs = [P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"] * c / S,
                         impedance=0) for c in currents]
    b = V.BunchBatch(ctx, descs, [z])
    m = len(currents)
    b.set_csr([zr], [0] * m, [p["fc"]] * m, [P.C / p["bl"]] * m,
              every=1, capacity=8)
    return b


def uneven_batch(ctx):
    """The uneven batch (uneven_workload's seed 4: 96 bunches, 2000 steps
    per period) with one impedance per mesh size; also its (parameters,
    order) list and sizes."""
    from inovesa_gb300 import params as P
    from inovesa_gb300 import vfps as V
    ps, keys = uneven_workload(4, 96, 2000)
    zs = {}
    for k in keys:
        pk = next(p for p, _ in ps if p["ps_bins"] == k)
        zs[k] = V.makeImpedance(ctx, **P.wake_impedance_args(pk))
    descs = [P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"],
                         impedance=keys.index(p["ps_bins"]), it=it)
             for p, it in ps]
    return V.BunchBatch(ctx, descs, [zs[k] for k in keys]), ps, keys


def config_bursting(ctx, stream, hbm):
    """Bursting: 512x512, parallel-plates CSR (g/R = 0.006) + resistive
    wall (5.8e7 S/m), 4000 steps per period, S = 1.2, CSR power every step:
    the plain GPU loop (C++ driver), the batched step on that bunch and on
    a 32-bunch bursting scan (S 0.8..1.6), all with the CSR power of every
    bunch every step; densities against FP64 after 200 steps."""
    import oracle
    from inovesa_gb300 import params as P
    p, z, zr = bursting_params(ctx)
    S = p["S_csr"]
    total, warm = 200, 20
    rate, dens = plain_driver(p, 0, 4, False, total - warm, warm, csr=True)
    d = P.fill_desc(oracle.BunchDesc(), p, 0, Ib=p["Ib"], it=4)
    ref = oracle.Sim([d], Z=z.data(), dtype=np.float64)
    ref.step(total)
    out = {"workload": "bursting 512x512, parallel-plates CSR g/R=0.006 + "
                       "resistive wall, 4000 steps/period, S=1.2, CSR power "
                       "every step",
           "gpu_plain": rate,
           "gpu_plain_driver": "C++ (include/vfps.hpp), one map per launch",
           "plain_density_l1_vs_fp64": rel_l1(dens, ref.density(0)),
           "accuracy_steps": total}

    def batch(currents):
        return bursting_batch(ctx, p, z, zr, currents)
    b1 = batch([S])
    out["gpu_batched_one"] = timed_batch(b1, stream, 200, 10)
    bs = batch(list(np.geomspace(0.8, 1.6, 32)))
    out["gpu_batched_scan32"] = timed_batch(bs, stream, 100, 5)
    kt = bs.kernel_times(20)
    out["scan32_kernel_ms_per_step"] = kt
    out["scan32_maps_hbm_frac"] = 8.0 * bs.cells / (kt["k_bmaps0"] / 1e3) \
        / 1e9 / hbm
    b3 = batch([S])
    b3.step(total)
    out["batched_density_l1_vs_fp64"] = rel_l1(b3.density(0),
                                               ref.density(0))
    out["cpu_1core"], k1 = cpu_rate([d], z.data(), 3.0, 1)
    out["cpu_sample"] = "%d solver steps, 1 thread" % k1
    return out


def config_uneven(ctx, stream, hbm, cores):
    """Uneven batch: 96 seeded bunches of 128..1024 rows, S ~ U(0.1, 1.5),
    orders 2..4, 2000 steps per period (38.5 M cells per step, larger than
    L2): batched rate, per-kernel times, the chain-0 maps' HBM fraction,
    the plain loop (C++ driver, one bunch of each size, weighted by the
    batch's mix), a host-core sample."""
    from inovesa_gb300 import params as P
    b, ps, keys = uneven_batch(ctx)
    sizes = np.array([p["ps_bins"] for p, _ in ps])
    out = {"workload": "uneven batch: 96 bunches, meshes 128..1024 "
                       "(seeded), S~U(0.1,1.5), orders 2..4, 2000 "
                       "steps/period",
           "cells_per_step": int(b.cells),
           "gpu_batched": timed_batch(b, stream, 50, 5)}
    kt = b.kernel_times(20)
    out["kernel_ms_per_step"] = kt
    out["maps_hbm_frac"] = 8.0 * b.cells / (kt["k_bmaps0"] / 1e3) / 1e9 / hbm
    rates = {}
    for k in keys:
        i = int(np.nonzero(sizes == k)[0][0])
        p, it = ps[i]
        rates[k], _ = plain_driver(p, 0, it, False, 100, 10)
    t_plain = sum(int(n) ** 2 / rates[int(n)] for n in sizes)
    out["gpu_plain"] = b.cells / t_plain
    out["gpu_plain_driver"] = ("C++ (include/vfps.hpp), one bunch of each "
                               "size, weighted by the batch")
    import oracle
    od = [P.fill_desc(oracle.BunchDesc(), p, 0, Ib=p["Ib"], it=it)
          for p, it in ps[:max(cores, 1)]]
    out["cpu_all_cores"], kk = cpu_rate(od, None, 4.0, cores)
    out["cpu_sample"] = ("%d bunches of the batch, %d steps, no wake, %d "
                         "threads" % (len(od), kk, cores))
    return out


def config_warm_start(ctx):
    """Learned warm start on 256x256 bunches: the network trained on 512
    solver equilibria (S ~ U(0.02, 0.45), g/R in 0.004..0.008, damping 5..150
    synchrotron periods), then periods to equilibrium (profile change below
    1e-5 per period for three periods, the solver judging) of 24 held-out
    bunches from the Gaussian start, from the potential-well state alone
    and from the proposal; and of 24 more at a damping time of 100 periods
    (the plain single-bunch workload's)."""
    from inovesa_gb300 import warmstart as W
    t = time.perf_counter()
    res, _ = W.experiment(ctx, n=256, spt=1000, ntrain=512, ntest=24,
                          iters=2000, max_periods=600, seed=11,
                          report_damping=(100.0,))
    res["seconds"] = time.perf_counter() - t
    return res


def rotation_scan_batch(ctx, p, currents, z):
    """The headline's current scan on the rotation chain (chain 1)."""
    from inovesa_gb300 import params as P
    from inovesa_gb300 import vfps as V
    descs = [P.fill_desc(V.BunchDesc(), p, 1, Ib=float(ib), impedance=0)
             for ib in currents]
    return V.BunchBatch(ctx, descs, [z])


def config_scan_rotation(ctx, stream, hbm, p, currents, z):
    """The current scan of the headline on the rotation chain (cubic
    RotationMap, wake kick, Fokker-Planck; the batched k_bmaps1): rate,
    kernel times and the maps kernel's HBM fraction."""
    b = rotation_scan_batch(ctx, p, currents, z)
    out = {"workload": "the headline's 256-bunch scan on the rotation "
                       "chain (cubic RotationMap, wake kick, "
                       "Fokker-Planck)",
           "gpu_batched": timed_batch(b, stream, 50, 5)}
    kt = b.kernel_times(20)
    out["kernel_ms_per_step"] = kt
    out["maps_hbm_frac"] = 8.0 * b.cells / (kt["k_bmaps1"] / 1e3) / 1e9 / hbm
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=16)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other workloads of the benchmark plan "
                         "(the \"configs\" key)")
    ap.add_argument("--wake-mode", type=int, default=0, choices=[0, 1],
                    help="wake potentials on the CUDA cores (0) or the "
                         "tensor cores (1); the other mode is measured "
                         "alongside")
    ap.add_argument("--profile", action="store_true",
                    help="timed steps only (for ncu): no e2e, plain loop or "
                         "CPU legs")
    ap.add_argument("--workload", default="scan",
                    choices=["scan", "uneven", "bursting32", "rotation"],
                    help="with --profile: the batch stepped (the current "
                         "scan, the uneven 96-bunch batch, the 32-bunch "
                         "512x512 bursting scan or the current scan on the "
                         "rotation chain)")
    args = ap.parse_args()
    if args.profile:
        args.no_cpu = True
        args.no_configs = True
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    import __graft_entry__
    __graft_entry__.build()
    from inovesa_gb300 import _lib
    from inovesa_gb300 import params as P
    from inovesa_gb300 import vfps as V

    p, gap, currents = workload_params()
    ctx = V.Context(local)
    if args.profile and args.workload == "uneven":
        batch, _, _ = uneven_batch(ctx)
    elif args.profile and args.workload == "rotation":
        z = V.makeImpedance(ctx, **P.wake_impedance_args(p))
        batch = rotation_scan_batch(ctx, p, currents, z)
    elif args.profile and args.workload == "bursting32":
        batch = bursting_batch(ctx, *bursting_params(ctx),
                               list(np.geomspace(0.8, 1.6, 32)))
    else:
        z = V.makeImpedance(ctx, **P.wake_impedance_args(p))
        batch = make_batch(ctx, p, currents, z)
        batch.set_wake_mode(args.wake_mode)
    cells = batch.cells
    stream = torch.cuda.ExternalStream(
        _lib.lib().vfps_stream(ctx.handle), device=local)

    launches_per_step, tile_rows = batch.info()
    # L2 is flushed before every timed step by overwriting a buffer twice
    # its size (outside the timed events): the two density buffers of the
    # workload together are about as large as L2
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32,
                        device="cuda:%d" % local)

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)

    start = batch.download()   # the Gaussian start (accuracy check)
    batch.step(args.warmup)
    ctx.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if args.profile:
        # the timed steps are the profiled range (ncu --profile-from-start
        # off skips the set-up and the tile-size tuning)
        torch.cuda.profiler.start()
    with ClockSampler(local) as clk:
        for e0, e1 in ev:
            flush_l2()
            e0.record(stream)
            batch.step(1)
            e1.record(stream)
        ev[-1][1].synchronize()
    if args.profile:
        torch.cuda.profiler.stop()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    torch.cuda.synchronize()
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    total_cells = cells * args.steps * world
    value = total_cells / (ms / 1e3)
    ms_step = ms / args.steps
    status = ctx.device_status()
    if status != 0:
        print(json.dumps({"error": "device status %d after the timed steps"
                          % status}), flush=True)
        sys.exit(3)
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_run": True,
                              "workload": args.workload, "value": value,
                              "ms_per_step": ms_step,
                              "tile_rows": tile_rows,
                              "kernel_tiles": batch.kernel_tiles()}),
                  flush=True)
        return

    # back-to-back steps (8-step graphs, no flush): what a long run sees
    c0 = torch.cuda.Event(enable_timing=True)
    c1 = torch.cuda.Event(enable_timing=True)
    c0.record(stream)
    batch.step(args.steps)
    c1.record(stream)
    c1.synchronize()
    continuous = cells * args.steps / (c0.elapsed_time(c1) / 1e3)

    # per-kernel durations after an L2 flush (CUDA events on the
    # library's stream between the kernels of a step)
    kt = {}
    nk = 32
    for _ in range(nk):
        flush_l2()
        for k, v in batch.kernel_times(1).items():
            kt[k] = kt.get(k, 0.0) + v / nk

    # the other wake mode: kernel times and back-to-back steps
    other = 1 - args.wake_mode
    batch.set_wake_mode(other)
    batch.step(8)
    kt_o = {}
    for _ in range(nk):
        flush_l2()
        for k, v in batch.kernel_times(1).items():
            kt_o[k] = kt_o.get(k, 0.0) + v / nk
    o0 = torch.cuda.Event(enable_timing=True)
    o1 = torch.cuda.Event(enable_timing=True)
    o0.record(stream)
    batch.step(args.steps)
    o1.record(stream)
    o1.synchronize()
    other_cont = cells * args.steps / (o0.elapsed_time(o1) / 1e3)
    batch.set_wake_mode(args.wake_mode)
    if ctx.device_status() != 0:
        print(json.dumps({"error": "device status after the wake-mode run"}),
              flush=True)
        sys.exit(3)

    # end to end through the C ABI with pinned host buffers: each call is
    # one output interval of the reference (100 solver steps): density in,
    # steps, density, profiles and fillings out
    nbytes = cells * 4
    hin = C.c_void_p()
    hout = C.c_void_p()
    L = _lib.lib()
    _lib.check(L.vfps_host_alloc(ctx.handle, nbytes, C.byref(hin)))
    _lib.check(L.vfps_host_alloc(ctx.handle, nbytes, C.byref(hout)))
    a_in = np.ctypeslib.as_array((C.c_float * cells).from_address(hin.value))
    a_out = np.ctypeslib.as_array((C.c_float * cells).from_address(hout.value))
    a_in[:] = batch.download()
    hprof = C.c_void_p()
    hfill = C.c_void_p()
    _lib.check(L.vfps_host_alloc(ctx.handle, batch.rows * 4, C.byref(hprof)))
    _lib.check(L.vfps_host_alloc(ctx.handle, NB * 4, C.byref(hfill)))
    prof = np.ctypeslib.as_array(
        (C.c_float * batch.rows).from_address(hprof.value))
    fill = np.ctypeslib.as_array((C.c_float * NB).from_address(hfill.value))
    batch.run(a_in, args.e2e_steps, a_out, prof, fill)
    reps = max(3, 2000 // args.e2e_steps)
    t = time.perf_counter()
    for _ in range(reps):
        batch.run(a_in, args.e2e_steps, a_out, prof, fill)
    e2e_s = (time.perf_counter() - t) / reps
    e2e_value = cells * args.e2e_steps * world / e2e_s
    del a_in, a_out, prof, fill
    for h in (hin, hout, hprof, hfill):
        _lib.check(L.vfps_host_free(ctx.handle, h))

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # plain one-map-per-launch loop, one bunch at a time (the C++ driver:
    # the reference's loop over include/vfps.hpp)
    plain_value, _ = plain_driver(p, 0, 4, False, 1000, 20,
                                  Ib=float(currents[NB // 2]))
    hbm, peak_kind = peaks()
    # dominant kernel: the fused maps of chain 0 (reads and writes every
    # density cell once: 8 algorithmic bytes per cell)
    ms_maps = kt["k_bmaps0"]
    achieved = 8.0 * cells / (ms_maps / 1e3) / 1e9
    tpc = traffic_per_cell()
    cfg = config_dict(p, gap, "flushed before every timed step (fill of a "
                      "%d MiB buffer outside the timed events)"
                      % (2 * L2_BYTES // 2 ** 20))
    cfg["tile_rows"] = tile_rows
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (Gaussian start, seeded log-spaced currents)",
        "config": cfg,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": 8 * cells,
                     "traffic": None if tpc is None else tpc * cells,
                     "kernel": ("k_bmaps0f<128, 256>"
                                if batch.kernel_tiles()["k_bmaps0f"] > 0
                                else "k_bmaps0"),
                     "kernel_ms": ms_maps},
        "kernel_ms_per_step": kt,
        "continuous_value": continuous,
        "wake_mode": ["cuda cores", "tensor cores"][args.wake_mode],
        "other_wake_mode": {
            "wake_mode": ["cuda cores", "tensor cores"][other],
            "kernel_ms_per_step": kt_o, "continuous_value": other_cont},
        "e2e": {"value": e2e_value, "unit": "cell-updates/s",
                "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes + batch.rows * 4 + NB * 4,
                "step": "one output interval of %d solver steps (the "
                        "reference's default outstep is 100)"
                        % args.e2e_steps,
                "call": "vfps_batch_run (pinned host density in, solver "
                        "steps, density/profiles/filling out)"},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clk.summary(),
        "plain_loop": {"value": plain_value, "unit": "cell-updates/s",
                       "driver": "C++ (include/vfps.hpp), one map per "
                                 "launch, one bunch of the scan"},
        "batched_over_plain": value / plain_value,
    }
    if not args.no_cpu:
        zh = z.data()
        line["cpu_baseline"] = cpu_baseline(p, currents, zh)
        line["accuracy"] = accuracy_check(batch, start, p, currents, zh,
                                          os.cpu_count() or 1)
    if not args.no_configs and world == 1:
        # the other workloads of the benchmark plan (not the headline)
        cores = os.cpu_count() or 1
        t_cfg = time.perf_counter()
        cfgs = {}
        for key, fn in (
                ("plain_256_rotation",
                 lambda: config_plain_rotation(ctx, hbm)),
                ("bursting_512", lambda: config_bursting(ctx, stream, hbm)),
                ("uneven_96", lambda: config_uneven(ctx, stream, hbm, cores)),
                ("scan_rotation_chain",
                 lambda: config_scan_rotation(ctx, stream, hbm, p, currents,
                                              z)),
                ("warm_start_256", lambda: config_warm_start(ctx))):
            try:
                cfgs[key] = fn()
            except Exception as e:   # reported, the headline stands
                cfgs[key] = {"error": repr(e)[:300]}
        cfgs["seconds"] = time.perf_counter() - t_cfg
        line["configs"] = cfgs
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
