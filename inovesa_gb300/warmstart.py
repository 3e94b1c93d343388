"""Learned warm start: the equilibrium density of a bunch proposed from
its normalised current S, gap ratio g/R and damping time (in synchrotron
periods).  The proposal is the potential-well state of the bunch's step
(vfps_batch_potential_well: the Haissinski solution written in the
invariant of the discrete kick-drift step, computed on the device) plus a
correction that a small network predicts, trained on the difference
between equilibria this solver produced and that state.

The proposal enters the solver as initial data (the reference's
PhaseSpace data argument, inc/PS/PhaseSpace.hpp:54-61, the hook of
InitialDistFile in src/main.cpp:469-525); the solver decides whether a
start was good: a bunch counts as converged when the relative L1 change of its profile over
one synchrotron period falls below a tolerance, and the warm-started and
the Gaussian-started runs must reach the same equilibrium.

Forward, backward and Adam steps are the library's own kernels
(vfps_ws_forward / vfps_ws_backward / vfps_ws_adam); PyTorch only holds
the device buffers.
"""
import ctypes as C
import math

import numpy as np

from . import _lib
from . import params as P
from . import vfps as V

NIN, NH, NLAT = 3, 128, 32
GAP_LO, GAP_HI = 0.004, 0.008
# damping times of the training domain, in synchrotron periods: from
# strongly damped rings to the reference's default lattice (about 135
# periods at 1000 steps per period) and the 100 periods of the plain
# single-bunch workload
TD_LO, TD_HI = 5.0, 150.0


def normalise_inputs(S, gap_ratio, damping_periods):
    """Network inputs, each about unit range over the training domain (the
    damping time on a log scale)."""
    lo, hi = math.log(TD_LO), math.log(TD_HI)
    td = np.log(np.asarray(damping_periods, np.float64))
    return np.stack([np.asarray(S, np.float64) / 0.25 - 1.0,
                     (np.asarray(gap_ratio, np.float64) - 0.006) / 0.002,
                     (2.0 * td - (lo + hi)) / (hi - lo)],
                    axis=-1).astype(np.float32)


def bunch_params(n, spt, S, gap_ratio, damping_periods):
    """Derived parameters of one bunch (parallel-plates CSR impedance)."""
    base = P.derive(GridSize=n, StepsPerTs=spt, padding=2.0)
    gap = gap_ratio * base["R_bend"]
    return P.derive(GridSize=n, StepsPerTs=spt, padding=2.0, VacuumGap=gap,
                    S_csr=float(S), DampingTime=damping_periods / base["fs"])


# a bunch counts as at equilibrium once the profile change has stayed below
# the tolerance for this many periods in a row (the profile is sampled
# once per synchrotron period, and a coherent oscillation can make a
# single sample look still)
CONFIRM = 3


def run_to_equilibrium(ctx, samples, n=256, spt=1000, tol=1e-5,
                       max_periods=400, start=None, confirm=CONFIRM):
    """Advance one batch of bunches period by period until the relative L1
    change of each profile over a period has been below tol for `confirm`
    periods in a row.

    samples: (S, gap ratio, damping periods) per bunch; start: initial
    densities [nb][n][n], "potential_well" (the device's potential-well
    state) or None (the Gaussian).  Returns (final densities [nb][n][n],
    periods to equilibrium per bunch: the first period of the run of
    `confirm` quiet periods (-1: not converged))."""
    zs, keys, descs = {}, [], []
    for S, g, td in samples:
        p = bunch_params(n, spt, S, g, td)
        k = round(float(g), 9)
        if k not in zs:
            zs[k] = V.makeImpedance(ctx, **P.wake_impedance_args(p))
            keys.append(k)
        descs.append(P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"],
                                 impedance=keys.index(k)))
    b = V.BunchBatch(ctx, descs, [zs[k] for k in keys])
    nb = len(samples)
    lay = [b.layout(i) for i in range(nb)]
    if isinstance(start, str):
        if start != "potential_well":
            raise ValueError("unknown start " + start)
        b.potential_well()
    elif start is not None:
        full = b.download()
        for i in range(nb):
            off = lay[i][0]
            full[off:off + n * n] = np.asarray(start[i], np.float32).ravel()
        b.upload(full)
    done = np.full(nb, -1)

    def profiles():
        pr = b.profiles()
        return np.stack([pr[lay[i][1]:lay[i][1] + n] for i in range(nb)])

    prev = profiles()
    streak = np.zeros(nb, int)
    for period in range(1, max_periods + 1):
        b.step(spt)
        cur = profiles()
        change = (np.abs(cur - prev).sum(1)
                  / np.maximum(np.abs(cur).sum(1), 1e-30))
        streak = np.where(change < tol, streak + 1, 0)
        newly = (done < 0) & (streak >= confirm)
        done[newly] = period - confirm + 1
        prev = cur
        if np.all(done >= 0):
            break
    if ctx.device_status() != 0:
        raise RuntimeError("device error status during the equilibrium run")
    full = b.download()
    dens = np.stack([full[lay[i][0]:lay[i][0] + n * n].reshape(n, n)
                     for i in range(nb)])
    return dens, done


def potential_well_states(ctx, samples, n=256, spt=1000, chunk=256):
    """The device's potential-well state of every bunch, [nb][n][n]."""
    out = []
    for i in range(0, len(samples), chunk):
        d, _ = run_to_equilibrium(ctx, samples[i:i + chunk], n=n, spt=spt,
                                  max_periods=0, start="potential_well")
        out.append(d)
    return np.concatenate(out)


def simpson_normalise(d, delta):
    """Scale densities to unit Simpson integral (weights of the reference,
    src/PS/PhaseSpace.cpp:486-501); negative cells are set to zero."""
    d = np.maximum(np.asarray(d, np.float64), 0.0)
    n = d.shape[-1]
    w = np.full(n, 2.0)
    w[1::2] = 4.0
    w[0] = w[-1] = 1.0
    w *= delta / 3.0
    integral = np.einsum("...xy,x,y->...", d, w, w)
    return (d / integral[..., None, None]).astype(np.float32)


class WarmStartNet:
    """The network, its FP32 masters, BF16 copies, gradients and Adam
    moments, all on one CUDA device."""

    def __init__(self, ctx, npix, seed=0, device=0):
        import torch
        self.torch = torch
        self.ctx = ctx
        self.npix = int(npix)
        self.dev = torch.device("cuda", device)
        rng = np.random.default_rng(seed)
        shapes = {"w1": (NH, NIN), "b1": (NH,), "w2": (NH, NH), "b2": (NH,),
                  "w3": (NLAT, NH), "b3": (NLAT,), "wd": (NLAT, self.npix),
                  "bd": (self.npix,)}
        self.names = list(shapes)
        self.w, self.g, self.m, self.v, self.w16 = {}, {}, {}, {}, {}
        for k, shp in shapes.items():
            if k.startswith("w"):
                fan_in = shp[1] if k != "wd" else NLAT
                init = rng.normal(0.0, 1.0 / math.sqrt(fan_in), size=shp)
                if k == "wd":
                    init *= 1e-3
            else:
                init = np.zeros(shp)
            self.w[k] = torch.tensor(init, dtype=torch.float32,
                                     device=self.dev)
            self.g[k] = torch.zeros(shp, dtype=torch.float32, device=self.dev)
            self.m[k] = torch.zeros(shp, dtype=torch.float32, device=self.dev)
            self.v[k] = torch.zeros(shp, dtype=torch.float32, device=self.dev)
            if k.startswith("w"):
                self.w16[k] = self.w[k].to(torch.bfloat16)
        self.step_count = 0
        self._ws = {}

    def set_bias(self, mean_density):
        """Start the decoder from the mean training density."""
        self.w["bd"].copy_(self.torch.as_tensor(
            np.asarray(mean_density, np.float32).ravel(), device=self.dev))

    def _net(self, grad=False):
        src = self.g if grad else None
        f = {}
        for k in self.names:
            if grad:
                f[k] = src[k].data_ptr()
            elif k.startswith("w"):
                f[k] = self.w16[k].data_ptr()
            else:
                f[k] = self.w[k].data_ptr()
        return _lib.WsNet(NIN, NH, NLAT, self.npix, f["w1"], f["b1"],
                          f["w2"], f["b2"], f["w3"], f["b3"], f["wd"],
                          f["bd"])

    def _work(self, B):
        if B not in self._ws:
            t, d = self.torch, self.dev
            self._ws[B] = {
                "h1": t.zeros(B, NH, device=d), "h2": t.zeros(B, NH, device=d),
                "z": t.zeros(B, NLAT, device=d),
                "y": t.zeros(B, self.npix, device=d),
                "g": t.zeros(B, self.npix, device=d),
                "dz": t.zeros(B, NLAT, device=d),
                "d1": t.zeros(B, NH, device=d), "d2": t.zeros(B, NH, device=d),
                "lp": t.zeros(256, dtype=t.float64, device=d)}
        return self._ws[B]

    def _x(self, x):
        return self.torch.as_tensor(np.ascontiguousarray(x, np.float32),
                                    device=self.dev)

    def forward(self, x):
        """Densities [B][npix] (host) for normalised inputs x [B][3]."""
        xt = self._x(x)
        B = xt.shape[0]
        w = self._work(B)
        self.torch.cuda.synchronize(self.dev)
        net = self._net()
        _lib.check(_lib.lib().vfps_ws_forward(
            self.ctx.handle, C.byref(net), xt.data_ptr(), B,
            w["h1"].data_ptr(), w["h2"].data_ptr(), w["z"].data_ptr(),
            w["y"].data_ptr(), None, None, None, 0), self.ctx.handle)
        self.ctx.synchronize()
        return w["y"].cpu().numpy().copy()

    def train_step(self, x, target, lr=1e-3):
        """One Adam step on a minibatch (target [B][npix] on the device or
        host); returns the loss."""
        t = self.torch
        xt = self._x(x)
        tt = t.as_tensor(target, dtype=t.float32, device=self.dev)
        B = xt.shape[0]
        w = self._work(B)
        t.cuda.synchronize(self.dev)
        L = _lib.lib()
        net, grad = self._net(), self._net(grad=True)
        nparts = 256
        _lib.check(L.vfps_ws_forward(
            self.ctx.handle, C.byref(net), xt.data_ptr(), B,
            w["h1"].data_ptr(), w["h2"].data_ptr(), w["z"].data_ptr(), None,
            tt.data_ptr(), w["g"].data_ptr(), w["lp"].data_ptr(), nparts),
            self.ctx.handle)
        _lib.check(L.vfps_ws_backward(
            self.ctx.handle, C.byref(net), C.byref(grad), xt.data_ptr(), B,
            w["h1"].data_ptr(), w["h2"].data_ptr(), w["z"].data_ptr(),
            w["g"].data_ptr(), w["dz"].data_ptr(), w["d1"].data_ptr(),
            w["d2"].data_ptr()), self.ctx.handle)
        self.step_count += 1
        for k in self.names:
            w16 = self.w16[k].data_ptr() if k in self.w16 else None
            _lib.check(L.vfps_ws_adam(
                self.ctx.handle, self.w[k].data_ptr(), self.g[k].data_ptr(),
                self.m[k].data_ptr(), self.v[k].data_ptr(), w16,
                self.w[k].numel(), lr, 0.9, 0.999, 1e-8, self.step_count),
                self.ctx.handle)
        self.ctx.synchronize()
        return float(w["lp"].sum().item()) / (B * self.npix)

    def gradients(self, x, target):
        """Loss and gradients (host arrays) without an update (for checks)."""
        t = self.torch
        xt = self._x(x)
        tt = t.as_tensor(target, dtype=t.float32, device=self.dev)
        B = xt.shape[0]
        w = self._work(B)
        t.cuda.synchronize(self.dev)
        L = _lib.lib()
        net, grad = self._net(), self._net(grad=True)
        _lib.check(L.vfps_ws_forward(
            self.ctx.handle, C.byref(net), xt.data_ptr(), B,
            w["h1"].data_ptr(), w["h2"].data_ptr(), w["z"].data_ptr(),
            w["y"].data_ptr(), tt.data_ptr(), w["g"].data_ptr(),
            w["lp"].data_ptr(), 256), self.ctx.handle)
        _lib.check(L.vfps_ws_backward(
            self.ctx.handle, C.byref(net), C.byref(grad), xt.data_ptr(), B,
            w["h1"].data_ptr(), w["h2"].data_ptr(), w["z"].data_ptr(),
            w["g"].data_ptr(), w["dz"].data_ptr(), w["d1"].data_ptr(),
            w["d2"].data_ptr()), self.ctx.handle)
        self.ctx.synchronize()
        loss = float(w["lp"].sum().item()) / (B * self.npix)
        return loss, {k: self.g[k].cpu().numpy().copy() for k in self.names}

    def weights_bf16(self):
        """The weights the kernels use (BF16 rounded), as float64 arrays."""
        out = {}
        for k in self.names:
            src = self.w16[k] if k in self.w16 else self.w[k]
            out[k] = src.float().cpu().numpy().astype(np.float64)
        return out


def train(net, x, targets, iters=2000, batch=64, lr=1e-3, seed=1):
    """Minibatch Adam on (x, targets); cosine-decayed learning rate.
    Returns the loss history."""
    rng = np.random.default_rng(seed)
    t = net.torch
    tg = t.as_tensor(np.asarray(targets, np.float32).reshape(len(x), -1),
                     device=net.dev)
    hist = []
    for it in range(iters):
        idx = rng.choice(len(x), size=min(batch, len(x)), replace=False)
        rate = lr * 0.5 * (1 + math.cos(math.pi * it / iters)) + lr * 1e-3
        it_idx = t.as_tensor(idx, device=net.dev)
        hist.append(net.train_step(x[idx], tg[it_idx].contiguous(), rate))
    return hist


def sample_inputs(rng, count, quantise_gap, damping=None):
    """(S, gap ratio, damping periods) drawn from the training domain (S
    and g/R uniform, the damping time log-uniform, or fixed to `damping`);
    training gaps sit on a grid of 9 values (one impedance each)."""
    S = rng.uniform(0.02, 0.45, size=count)
    g = rng.uniform(GAP_LO, GAP_HI, size=count)
    if quantise_gap:
        g = np.round(g / 0.0005) * 0.0005
    if damping is None:
        td = np.exp(rng.uniform(math.log(TD_LO), math.log(TD_HI),
                                size=count))
    else:
        td = np.full(count, float(damping))
    return list(zip(S.tolist(), g.tolist(), td.tolist()))


def equilibria(ctx, samples, n, spt, tol, max_periods, start=None,
               chunk=256):
    dens, done = [], []
    for i in range(0, len(samples), chunk):
        d, p = run_to_equilibrium(
            ctx, samples[i:i + chunk], n=n, spt=spt, tol=tol,
            max_periods=max_periods,
            start=start if start is None or isinstance(start, str)
            else start[i:i + chunk])
        dens.append(d)
        done.append(p)
    return np.concatenate(dens), np.concatenate(done)


def evaluate(ctx, net, test_in, scale, n, spt, tol, max_periods, dq):
    """Periods to equilibrium of held-out inputs from the Gaussian start,
    from the potential-well state alone and from the proposal (state plus
    the learned correction), judged by the solver; the end states of the
    warm and the Gaussian runs compared."""
    ntest = len(test_in)
    g_d, g_p = equilibria(ctx, test_in, n, spt, tol, max_periods)
    base = potential_well_states(ctx, test_in, n, spt)
    _, h_p = equilibria(ctx, test_in, n, spt, tol, max_periods,
                        start=base)
    corr = net.forward(normalise_inputs(*np.array(test_in).T))
    prop = simpson_normalise(base + scale * corr.reshape(-1, n, n), dq)
    w_d, w_p = equilibria(ctx, test_in, n, spt, tol, max_periods, start=prop)
    both = (g_p > 0) & (w_p > 0) & (h_p > 0)
    same = np.array([np.abs(w_d[i] - g_d[i]).sum() / np.abs(g_d[i]).sum()
                     for i in range(ntest)])
    ref = simpson_normalise(g_d, dq)

    def err(d):
        return np.array([np.abs(d[i] - ref[i]).sum() / np.abs(ref[i]).sum()
                         for i in range(ntest)])

    def med(v):
        return float(np.median(v)) if both.any() else None

    return {
        "test_samples": int(ntest), "test_converged_all": int(both.sum()),
        "test_converged_gaussian": int((g_p > 0).sum()),
        "test_converged_potential_well": int((h_p > 0).sum()),
        "test_converged_warm": int((w_p > 0).sum()),
        "periods_gaussian_median": med(g_p[both]),
        "periods_potential_well_median": med(h_p[both]),
        "periods_warm_median": med(w_p[both]),
        "speedup_potential_well_median":
            med(g_p[both] / np.maximum(h_p[both], 1)),
        "speedup_median": med(g_p[both] / np.maximum(w_p[both], 1)),
        "speedup_total": float(g_p[both].sum() / max(w_p[both].sum(), 1))
        if both.any() else None,
        "warm_faster_than_potential_well": int(
            (w_p[both] < h_p[both]).sum()),
        "warm_slower_than_potential_well": int(
            (w_p[both] > h_p[both]).sum()),
        "potential_well_l1_median": float(np.median(err(base))),
        "proposal_l1_median": float(np.median(err(prop))),
        "same_equilibrium_l1_max": float(same[both].max()) if both.any()
        else None,
        "same_equilibrium_l1_median": float(np.median(same[both]))
        if both.any() else None,
        # the same distance in units of a damping time's worth of the
        # stopping tolerance (the distance a run stopped by the rule may
        # still have to go, for each of the two runs)
        "same_equilibrium_per_damping_max": float(max(
            same[i] / (test_in[i][2] * tol) for i in range(ntest)
            if both[i])) if both.any() else None,
    }


def experiment(ctx, n=256, spt=1000, ntrain=2048, ntest=128, iters=3000,
               tol=1e-5, max_periods=300, seed=7, log=None, tol_train=None,
               max_periods_train=None, report_damping=()):
    """Train the correction on solver equilibria, then compare the periods
    to equilibrium on held-out inputs from the Gaussian, from the
    potential-well state alone and from the proposal (potential-well state
    plus the learned correction).  The training equilibria may be
    converged further than the judging tolerance (tol_train): the stopping
    rule samples the profile once per synchrotron period and leaves
    coherent oscillations of about a damping time's worth of the
    tolerance, which would otherwise be learned as noise.  report_damping:
    damping times (periods) with a held-out set of their own (S and g/R
    drawn as before), reported under "at_damping"."""
    rng = np.random.default_rng(seed)
    train_in = sample_inputs(rng, ntrain, True)
    test_in = sample_inputs(rng, ntest, False)
    axes = bunch_params(n, spt, *train_in[0])["axes"]
    dq = (axes[1] - axes[0]) / (n - 1)
    # training targets: equilibrium (unit charge) minus potential well
    tr_d, tr_p = equilibria(ctx, train_in, n, spt, tol_train or tol,
                            max_periods_train or max_periods,
                            start="potential_well")
    tr_base = potential_well_states(ctx, train_in, n, spt)
    ok = tr_p >= 0
    resid = (simpson_normalise(tr_d[ok], dq).astype(np.float64)
             - tr_base[ok]).reshape(int(ok.sum()), -1)
    scale = float(resid.std()) or 1.0
    x = normalise_inputs(*np.array(train_in)[ok].T)
    tgt = (resid / scale).astype(np.float32)
    net = WarmStartNet(ctx, n * n, seed=seed)
    net.set_bias(tgt.mean(0))
    hist = train(net, x, tgt, iters=iters)
    out = {
        "grid": n, "steps_per_period": spt, "tolerance_per_period": tol,
        "train_tolerance_per_period": tol_train or tol, "iters": iters,
        "damping_periods_domain": [TD_LO, TD_HI],
        "train_samples": int(ntrain), "train_converged": int(ok.sum()),
        "residual_scale": scale,
        "train_loss_first": hist[0], "train_loss_last": hist[-1],
    }
    out.update(evaluate(ctx, net, test_in, scale, n, spt, tol, max_periods,
                        dq))
    if report_damping:
        out["at_damping"] = {}
        for td in report_damping:
            held = sample_inputs(rng, ntest, False, damping=td)
            out["at_damping"][str(td)] = evaluate(
                ctx, net, held, scale, n, spt, tol, max_periods, dq)
    if log:
        log(out)
    return out, net


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description=experiment.__doc__)
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--steps-per-period", type=int, default=1000)
    ap.add_argument("--train", type=int, default=2048)
    ap.add_argument("--test", type=int, default=128)
    ap.add_argument("--iters", type=int, default=3000)
    ap.add_argument("--train-tol", type=float, default=None)
    ap.add_argument("--max-periods", type=int, default=600)
    ap.add_argument("--report-damping", type=float, nargs="*",
                    default=[100.0])
    a = ap.parse_args()
    from . import build as _build
    _build.build()
    c = V.Context(0)
    res, _ = experiment(c, n=a.grid, spt=a.steps_per_period, ntrain=a.train,
                        ntest=a.test, iters=a.iters, tol_train=a.train_tol,
                        max_periods=a.max_periods, max_periods_train=600,
                        report_damping=a.report_damping)
    print(json.dumps(res))
