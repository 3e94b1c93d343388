"""Plain solver loop: one map per launch, the reference's own sequence of
calls (src/main.cpp:469-760 for the set-up, :948-1053 for the step), for
one bunch or one multi-bunch beam (fillings per bunch, bucket numbers and
their spacing, src/main.cpp:248-321).  chain 0 is main.cpp's loop; chain 1
replaces the RF kick and drift by a RotationMap (the scheme of
test/TestRotationMap.cpp).
"""
from . import vfps as V


class PlainSolver:
    def __init__(self, ctx, p, chain=0, Ib=None, wake_impedance=None,
                 csr_impedance=None, it=None, clamp=False, data=None,
                 resume_step=None, fillings=None, buckets=None,
                 spacing=None):
        """data: initial density [n][n] or [nb][n][n] (else the Gaussian);
        with resume_step, data is a saved state that continues at that
        step (not normalised again, renormalisation schedule kept).
        fillings: each bunch's share of the charge (default one bunch);
        buckets, spacing: bucket numbers and mesh cells between buckets of
        a multi-bunch beam (default bucket 0, the derived spacing)."""
        o = p["opts"]
        self.p, self.chain = p, chain
        n = p["ps_bins"]
        it = int(o["InterpolationPoints"] if it is None else it)
        ib = p["Ib"] if Ib is None else Ib
        self.renormalize = int(o["RenormalizeCharge"])
        a = p["axes"]
        fill = [1.0] if fillings is None else [float(f) for f in fillings]
        self.buckets = [0] * len(fill) if buckets is None else list(buckets)
        spacing = p["spacing_bins"] if spacing is None else int(spacing)
        self.t1 = V.PhaseSpace(a[0], a[1], a[2], a[3], a[4], a[5], ctx,
                               ib / p["f_rev"], ib, fill,
                               o["InitialDistZoom"], data, n=n)
        if self.renormalize >= 0 and resume_step is None:
            self.t1.updateXProjection()
            self.t1.normalize()
        elif resume_step is not None:
            self.t1.updateXProjection()
        self.t2 = self.t1.copy()
        self.t3 = self.t1.copy()
        self.wake_field = None
        self.wkm = None
        if wake_impedance is not None:
            self.wake_field = V.ElectricField.wake(
                self.t1, wake_impedance, self.buckets, spacing, ctx,
                p["f_rev"], p["revolutionpart"], ib, p["E0"], p["sE"],
                p["dt"])
        if chain == 0:
            if o["LinearRF"]:
                self.rfm = V.RFKickMap(self.t2, self.t1, p["angle"],
                                       p["f_RF"], it, clamp)
            else:
                self.rfm = V.RFKickMap.sinusoidal(
                    self.t2, self.t1, p["revolutionpart"], p["V_eff"],
                    p["f_RF"], p["V0"], it, clamp)
            self.drm = V.DriftMap(self.t1, self.t3, p["slip"], p["E0"], it,
                                  clamp)
            if self.wake_field is not None:
                self.wkm = V.WakePotentialMap(self.t1, self.t2,
                                              self.wake_field, it, clamp)
                self.wm = self.wkm
            else:
                self.wm = V.Identity(self.t1, self.t2)
        else:
            self.rm = V.RotationMap(self.t1, self.t2, n, n, p["angle"], it,
                                    clamp, n * n if clamp else 0)
            if self.wake_field is not None:
                self.wkm = V.WakePotentialMap(self.t2, self.t3,
                                              self.wake_field, it, clamp)
                self.wm = self.wkm
            else:
                self.wm = V.Identity(self.t2, self.t3)
        if p["e1"] > 0:
            self.fpm = V.FokkerPlanckMap(self.t3, self.t1, n, n,
                                         int(o["FPType"]), int(o["FPTrack"]),
                                         p["e1"], int(o["derivation"]))
        else:
            self.fpm = V.Identity(self.t3, self.t1)
        self.rdtn = None
        if csr_impedance is not None:
            self.rdtn = V.ElectricField(self.t1, csr_impedance, self.buckets,
                                        0, ctx,
                                        p["f_rev"], p["revolutionpart"])
        self.simulationstep = 0 if resume_step is None else int(resume_step)

    def step(self, nsteps=1, csr=False):
        for _ in range(nsteps):
            if self.wkm is not None:
                self.wkm.update()
            if (self.renormalize > 0
                    and self.simulationstep % self.renormalize == 0):
                self.t1.integrateAndNormalize()
            else:
                self.t1.integrate()
            if csr and self.rdtn is not None:
                self.rdtn.updateCSR(self.p["fc"])
            if self.chain == 0:
                self.wm.apply()
                self.rfm.apply()
                self.drm.apply()
                self.fpm.apply()
            else:
                self.rm.apply()
                self.wm.apply()
                self.fpm.apply()
            self.t1.updateXProjection()
            self.simulationstep += 1

    def density(self, b=0):
        return self.t1.getData()[b]

    def profile(self, b=0):
        return self.t1.getProjection(0)[b]
