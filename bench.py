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

Prints one JSON line (rank 0).  --impl reference times the CPU
restatement of the reference solver loop (the oracle, float) on all host
cores on the same workload.
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
    path = os.path.join(ROOT, "profiles", "k_bmaps0_scan256.json")
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


def accuracy_check(got, p, currents, z, total_steps):
    """Density L1 of the batched FP32 result against the FP64 oracle for
    the lowest-current bunch over the whole run (bunches in the bursting
    regime are checked over short horizons by the tests: there FP32 and
    FP64 trajectories separate exponentially)."""
    import oracle
    from inovesa_gb300 import params as P
    out = {}
    i0 = 0
    d = P.fill_desc(oracle.BunchDesc(), p, 0, Ib=float(currents[i0]))
    ref = oracle.Sim([d], Z=z, dtype=np.float64)
    ref.step(total_steps, threads=1)
    want = ref.density(0)
    out["low_current_l1"] = float(np.abs(got - want).sum()
                                  / np.abs(want).sum())
    out["low_current_steps"] = int(total_steps)
    return out


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


def other_workload(args):
    """The other workloads of the benchmark plan, one JSON line each (not
    the headline): plain single bunch (256x256, cubic rotation chain, 500
    steps per period, free-space CSR, S = 0.05), bursting (512x512,
    parallel-plates CSR + resistive wall, 4000 steps per period, S = 1.2,
    CSR power every step), uneven batch (96 seeded bunches of 128..1024,
    orders 2..4, S ~ U(0.1, 1.5), 2000 steps per period)."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import oracle
    from inovesa_gb300 import params as P
    from inovesa_gb300 import vfps as V
    from inovesa_gb300.solver import PlainSolver
    ctx = V.Context(0)
    stream = torch.cuda.ExternalStream(
        __import__("inovesa_gb300._lib", fromlist=["lib"]).lib().vfps_stream(
            ctx.handle), device=0)
    cores = os.cpu_count() or 1
    out = {"workload": args.workload, "unit": "cell-updates/s",
           "metric": METRIC}

    def time_plain(s, n, steps, csr=False):
        s.step(10, csr=csr)
        ctx.synchronize()
        t = time.perf_counter()
        s.step(steps, csr=csr)
        ctx.synchronize()
        return n * n * steps / (time.perf_counter() - t)

    def time_oracle(descs, Z, seconds, threads):
        sim = oracle.Sim(descs, Z=Z, dtype=np.float32)
        t = time.perf_counter()
        sim.step(2, threads=threads)
        per = max((time.perf_counter() - t) / 2, 1e-4)
        k = max(2, int(seconds / per))
        t = time.perf_counter()
        sim.step(k, threads=threads)
        cells = sum(int(d.n) ** 2 for d in descs) * k
        return cells / (time.perf_counter() - t), k

    if args.workload in ("plain", "bursting"):
        if args.workload == "plain":
            n, spt, chain, S = 256, 500, 1, 0.05
            fs = P.derive(GridSize=n, StepsPerTs=spt)["fs"]
            p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                         VacuumGap=-1.0, S_csr=S, DampingTime=100.0 / fs)
            csr, clamp = False, True
        else:
            n, spt, chain, S = 512, 4000, 0, 1.2
            p0 = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0)
            p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                         VacuumGap=0.006 * p0["R_bend"], S_csr=S,
                         WallConductivity=5.8e7)
            csr, clamp = True, False
        z = V.makeImpedance(ctx, **P.wake_impedance_args(p))
        zr = (V.makeImpedance(ctx, **P.csr_impedance_args(p)) if csr
              else None)
        s = PlainSolver(ctx, p, chain=chain, wake_impedance=z,
                        csr_impedance=zr, it=4, clamp=clamp)
        out["gpu_plain"] = time_plain(s, n, args.steps, csr)
        d = P.fill_desc(oracle.BunchDesc(), p, chain, Ib=p["Ib"], it=4,
                        clamp=clamp)
        v1, k1 = time_oracle([d], z.data(), 10.0, 1)
        out["cpu_1core"] = v1
        out["cpu_sample"] = "%d solver steps of the bunch, 1 thread" % k1
        # accuracy of the plain GPU loop against FP64 over 2 periods
        s2 = PlainSolver(ctx, p, chain=chain, wake_impedance=z, it=4,
                         clamp=clamp)
        ref = oracle.Sim([d], Z=z.data(), dtype=np.float64)
        steps = 2 * spt if args.workload == "plain" else 200
        s2.step(steps)
        ref.step(steps)
        want = ref.density(0)
        out["density_l1_vs_fp64"] = float(
            np.abs(s2.density() - want).sum() / np.abs(want).sum())
        out["accuracy_steps"] = steps
        out["config"] = {"grid": n, "steps_per_period": spt, "S": S,
                         "chain": chain, "csr_every_step": csr}
        if args.workload == "bursting":
            # the batched step on the same bunch, and on a bursting scan of
            # 32 such bunches (S log-spaced 0.8..1.6), with every bunch's
            # CSR power recorded every step
            def batched(currents):
                descs = [P.fill_desc(V.BunchDesc(), p, 0,
                                     Ib=p["Ib"] * c / S, impedance=0)
                         for c in currents]
                b = V.BunchBatch(ctx, descs, [z])
                nbb = len(currents)
                b.set_csr([zr], [0] * nbb, [p["fc"]] * nbb,
                          [P.C / p["bl"]] * nbb, every=1, capacity=8)
                b.step(args.warmup)
                ctx.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                b.step(args.steps)
                e1.record(stream)
                e1.synchronize()
                return b, b.cells * args.steps / (e0.elapsed_time(e1) / 1e3)
            b1, out["gpu_batched_one"] = batched([S])
            _, out["gpu_batched_scan32"] = batched(
                list(np.geomspace(0.8, 1.6, 32)))
            b3, _ = batched([S])
            before = b3.download().reshape(n, n).copy()
            ref3 = oracle.Sim([d], Z=z.data(), data=before,
                              dtype=np.float64)
            b3.step(200)
            ref3.step(200)
            # shapes at equal charge (the oracle normalises the state it
            # is given; the batch's charge has drifted by ~1e-5 by then)
            want = ref3.density(0)
            got = b3.density(0).astype(np.float64)
            got *= want.sum() / got.sum()
            out["batched_density_l1_vs_fp64"] = float(
                np.abs(got - want).sum() / np.abs(want).sum())
            out["batched_note"] = ("batched rates include the CSR power of "
                                   "every bunch every step")
    else:
        rng = np.random.default_rng(4)
        nb, spt = 96, 2000
        sizes = rng.choice([128, 256, 512, 1024], size=nb)
        cur = rng.uniform(0.1, 1.5, size=nb)
        its = rng.choice([2, 3, 4], size=nb)
        keys = sorted(set(int(v) for v in sizes))
        zs = {}
        for k in keys:
            p0 = P.derive(GridSize=k, StepsPerTs=spt, padding=2.0)
            pk = P.derive(GridSize=k, StepsPerTs=spt, padding=2.0,
                          VacuumGap=0.006 * p0["R_bend"])
            zs[k] = V.makeImpedance(ctx, **P.wake_impedance_args(pk))
        descs, ps = [], []
        for n, S, it in zip(sizes, cur, its):
            n, it = int(n), int(it)
            p0 = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0)
            p = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0,
                         VacuumGap=0.006 * p0["R_bend"], S_csr=float(S))
            ps.append((p, it))
            descs.append(P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"],
                                     impedance=keys.index(n), it=it))
        b = V.BunchBatch(ctx, descs, [zs[k] for k in keys])
        b.step(args.warmup)
        ctx.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(args.steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out["gpu_batched"] = b.cells * args.steps / (ms / 1e3)
        out["kernel_ms_per_step"] = b.kernel_times(20)
        out["cells_per_step"] = int(sum(int(v) ** 2 for v in sizes))
        # the plain loop, one bunch at a time, on one bunch of each size
        rates = []
        for k in keys:
            i = int(np.nonzero(sizes == k)[0][0])
            p, it = ps[i]
            s = PlainSolver(ctx, p, chain=0, wake_impedance=zs[k], it=it)
            rates.append((k, time_plain(s, k, 200)))
        # whole batch one bunch after another at those rates
        t_plain = sum(int(n) ** 2 / dict(rates)[int(n)] for n in sizes)
        out["gpu_plain"] = out["cells_per_step"] / t_plain
        od = [P.fill_desc(oracle.BunchDesc(), p, 0, Ib=p["Ib"], it=it)
              for p, it in ps[:max(cores, 1)]]
        vv, kk = time_oracle(od, None, 12.0, cores)
        out["cpu_all_cores"] = vv
        out["cpu_cores"] = cores
        out["cpu_sample"] = ("%d bunches of the batch, %d steps, no wake, "
                             "%d threads" % (len(od), kk, cores))
        out["config"] = {"bunches": nb, "sizes": "seeded 128..1024",
                         "steps_per_period": spt}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=16)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="scan",
                    choices=["scan", "plain", "bursting", "uneven"],
                    help="scan: the headline line; the others print one "
                         "line of their own")
    ap.add_argument("--wake-mode", type=int, default=0, choices=[0, 1],
                    help="wake potentials on the CUDA cores (0) or the "
                         "tensor cores (1); the other mode is measured "
                         "alongside")
    ap.add_argument("--profile", action="store_true",
                    help="timed steps only (for ncu): no e2e, plain loop or "
                         "CPU legs")
    args = ap.parse_args()
    if args.profile:
        args.no_cpu = True
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != "scan":
        other_workload(args)
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
    from inovesa_gb300.solver import PlainSolver

    p, gap, currents = workload_params()
    ctx = V.Context(local)
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

    batch.step(args.warmup)
    ctx.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        for e0, e1 in ev:
            flush_l2()
            e0.record(stream)
            batch.step(1)
            e1.record(stream)
        ev[-1][1].synchronize()
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
    snap_low = batch.density(0)
    if args.profile:
        if rank == 0:
            print(json.dumps({"profile_run": True, "value": value,
                              "ms_per_step": ms_step}), flush=True)
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

    # plain one-map-per-launch loop, one bunch at a time
    plain = PlainSolver(ctx, p, chain=0, wake_impedance=z,
                        Ib=float(currents[NB // 2]))
    plain.step(20)
    ctx.synchronize()
    t = time.perf_counter()
    nplain = 300
    plain.step(nplain)
    ctx.synchronize()
    plain_value = GRID * GRID * nplain / (time.perf_counter() - t)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
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
                     "kernel": "k_bmaps0",
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
                       "driver": "Python, one map per launch"},
        "batched_over_plain": value / plain_value,
    }
    if not args.no_cpu:
        zh = z.data()
        line["cpu_baseline"] = cpu_baseline(p, currents, zh)
        line["accuracy"] = accuracy_check(snap_low, p, currents, zh,
                                          args.warmup + args.steps)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
