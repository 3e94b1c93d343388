"""Python mirror of the reference's solver-step classes over libvfps.

Names, argument order and error behaviour follow Inovesa's C++ classes
(PhaseSpace, RotationMap, KickMap, DriftMap, RFKickMap, FokkerPlanckMap,
Identity, WakePotentialMap, Impedance and its models, ElectricField), so
that code and tests written against those classes read the same.  The
``oclh`` argument of the reference becomes a :class:`Context` (one CUDA
device and stream).  Invalid set-ups raise :class:`InvalidArgument` (a
ValueError), as the reference raises std::invalid_argument.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import BunchDesc, InvalidArgument, VfpsError, check, lib

__all__ = [
    "Context", "PhaseSpace", "RotationMap", "KickMap", "DriftMap",
    "RFKickMap", "DynamicRFKickMap", "FokkerPlanckMap", "Identity",
    "WakePotentialMap",
    "Impedance", "FreeSpaceCSR", "ParallelPlatesCSR", "ResistiveWall",
    "ConstImpedance", "CollimatorImpedance", "makeImpedance",
    "ElectricField", "BunchBatch", "BunchDesc", "InvalidArgument",
    "VfpsError", "InterpolationType", "Axis", "FPType", "FPTracking",
    "DerivationType",
]


class InterpolationType:
    none, linear, quadratic, cubic = 1, 2, 3, 4


class Axis:
    x, y = 0, 1


class FPType:
    none, damping_only, diffusion_only, full = 0, 1, 2, 3


class FPTracking:
    none, approximation1, approximation2, stochastic = 0, 1, 2, 3


class DerivationType:
    two_sided, cubic = 3, 4


def _fptr(a):
    return a.ctypes.data_as(_lib.FP)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Context:
    """One CUDA device with one in-order stream (replaces the OpenCL
    handler)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        check(lib().vfps_create(C.byref(h), device))
        self._h = h

    @property
    def handle(self):
        return self._h

    def synchronize(self):
        check(lib().vfps_synchronize(self._h), self._h)

    def device_status(self):
        c = C.c_int()
        check(lib().vfps_device_status(self._h, C.byref(c)), self._h)
        return c.value

    def close(self):
        if getattr(self, "_h", None):
            lib().vfps_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Handle:
    _destroy = None

    def _check(self, rc):
        check(rc, self.ctx.handle)

    def close(self):
        h = getattr(self, "_h", None)
        if h:
            getattr(lib(), self._destroy)(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PhaseSpace(_Handle):
    """PhaseSpace(qmin, qmax, qscale, pmin, pmax, pscale, oclh, charge,
    current, filling={1}, zoom=1, data=None).

    The mesh size comes from the class-wide setSize(n, nb), like the
    reference's static sizes, unless ``n`` is given."""
    _destroy = "vfps_ps_destroy"
    _size = None

    @classmethod
    def setSize(cls, n, nb=1):
        cls._size = (int(n), int(nb))

    resetSize = setSize

    def __init__(self, qmin, qmax, qscale, pmin, pmax, pscale, oclh,
                 charge=1.0, current=1.0, filling=(1.0,), zoom=1.0,
                 data=None, n=None, _handle=None):
        self.ctx = oclh
        if _handle is not None:
            self._h = _handle
        else:
            if n is None:
                if PhaseSpace._size is None:
                    raise InvalidArgument(1, "mesh size not set")
                n = PhaseSpace._size[0]
            fill = _f32(filling)
            axes = (C.c_double * 6)(qmin, qmax, qscale, pmin, pmax, pscale)
            d = None if data is None else _f32(data)
            if d is not None and d.size != fill.size * n * n:
                raise InvalidArgument(1, "data has the wrong size")
            h = C.c_void_p()
            check(lib().vfps_ps_create(
                oclh.handle, fill.size, n, axes, charge, current, _fptr(fill),
                zoom, None if d is None else _fptr(d), C.byref(h)),
                oclh.handle)
            self._h = h
        nb, nn = C.c_uint32(), C.c_uint32()
        lib().vfps_ps_shape(self._h, C.byref(nb), C.byref(nn))
        self.nb, self.n = nb.value, nn.value
        self._filling_set = None if _handle is not None else _f32(filling)

    @property
    def handle(self):
        return self._h

    @property
    def nxy(self):
        return self.n * self.n

    def copy(self):
        h = C.c_void_p()
        self._check(lib().vfps_ps_copy(self._h, C.byref(h)))
        ps = PhaseSpace(0, 0, 0, 0, 0, 0, self.ctx, _handle=h)
        ps._filling_set = self._filling_set
        return ps

    __copy__ = copy

    def swap(self, other):
        self._check(lib().vfps_ps_swap(self._h, other._h))

    def assign(self, other):
        """operator=: copy the density of ``other``."""
        self._check(lib().vfps_ps_assign(self._h, other._h))
        return self

    def getData(self):
        out = np.empty((self.nb, self.n, self.n), np.float32)
        self._check(lib().vfps_ps_download(self._h, _fptr(out)))
        return out

    def setData(self, data):
        d = _f32(data)
        if d.size != self.nb * self.nxy:
            raise InvalidArgument(1, "data has the wrong size")
        self._check(lib().vfps_ps_upload(self._h, _fptr(d)))

    def devicePointer(self):
        return lib().vfps_ps_device_data(self._h)

    def _axis(self, axis):
        v = np.empty(self.n, np.float32)
        d, z = C.c_float(), C.c_float()
        self._check(lib().vfps_ps_axis(self._h, axis, _fptr(v), C.byref(d),
                                       C.byref(z)))
        return v, d.value, z.value

    def getAxis(self, axis):
        return self._axis(axis)[0]

    def getDelta(self, axis):
        return self._axis(axis)[1]

    def zerobin(self, axis):
        return self._axis(axis)[2]

    def q(self, x):
        return self.getAxis(0)[x]

    def p(self, y):
        return self.getAxis(1)[y]

    def updateXProjection(self):
        self._check(lib().vfps_ps_update_x_projection(self._h))

    def updateYProjection(self):
        self._check(lib().vfps_ps_update_y_projection(self._h))

    def integrate(self):
        self._check(lib().vfps_ps_integrate(self._h))

    def normalize(self):
        self._check(lib().vfps_ps_normalize(self._h))
        return self.getBunchPopulation()

    def integrateAndNormalize(self):
        self._check(lib().vfps_ps_integrate_and_normalize(self._h))
        return self.getBunchPopulation()

    def variance(self, axis):
        self._check(lib().vfps_ps_variance(self._h, axis))

    def getProjection(self, axis, bunch=None):
        out = np.empty((self.nb, self.n), np.float32)
        self._check(lib().vfps_ps_get_projection(self._h, axis, _fptr(out)))
        return out if bunch is None else out[bunch]

    def setProjection(self, axis, bunch, proj):
        p = _f32(proj)
        self._check(lib().vfps_ps_set_projection(self._h, axis, bunch,
                                                 _fptr(p)))

    def _filling(self):
        f = np.empty(self.nb, np.float32)
        tot = C.c_double()
        self._check(lib().vfps_ps_get_filling(self._h, _fptr(f),
                                              C.byref(tot)))
        return f, tot.value

    def getBunchPopulation(self):
        return self._filling()[0]

    def getSetBunchPopulation(self):
        return self._filling_set

    def getIntegral(self):
        return self._filling()[1]

    def _moments(self, axis):
        a = np.empty(self.nb, np.float32)
        v = np.empty(self.nb, np.float32)
        r = np.empty(self.nb, np.float32)
        self._check(lib().vfps_ps_get_moments(self._h, axis, _fptr(a),
                                              _fptr(v), _fptr(r)))
        return a, v, r

    def getMoment(self, axis, m):
        return self._moments(axis)[m]

    def getBunchLength(self):
        return self._moments(0)[2]

    def getEnergySpread(self):
        return self._moments(1)[2]


class SourceMap(_Handle):
    _destroy = "vfps_map_destroy"

    def __init__(self, grid_in, grid_out, handle):
        self.ctx = grid_in.ctx
        self._in, self._out = grid_in, grid_out
        self._h = handle

    def apply(self):
        self._check(lib().vfps_map_apply(self._h))

    def applyTo(self, pos):
        p = np.array(pos, dtype=np.float32).reshape(-1, 2).copy()
        self._check(lib().vfps_map_apply_to(self._h, _fptr(p), p.shape[0]))
        return p.reshape(np.shape(pos)) if np.ndim(pos) == 1 else p

    def applyToAll(self, particles):
        return self.applyTo(particles)


def _new_map(fn, grid_in, *args):
    h = C.c_void_p()
    check(fn(grid_in.handle, *args, C.byref(h)), grid_in.ctx.handle)
    return h


class RotationMap(SourceMap):
    """RotationMap(in, out, xsize, ysize, angle, it, interpol_clamped,
    rotmapsize)."""

    def __init__(self, grid_in, grid_out, xsize, ysize, angle, it,
                 interpol_clamped, rotmapsize, oclh=None):
        h = _new_map(lib().vfps_rotation_map_create, grid_in, grid_out.handle,
                     xsize, ysize, angle, it, int(interpol_clamped),
                     rotmapsize)
        super().__init__(grid_in, grid_out, h)


class KickMap(SourceMap):
    """KickMap(in, out, it, interpol_clamp, kd)."""

    def __init__(self, grid_in, grid_out, it, interpol_clamp, kd, oclh=None,
                 _handle=None):
        h = _handle if _handle is not None else _new_map(
            lib().vfps_kick_map_create, grid_in, grid_out.handle, it,
            int(interpol_clamp), kd)
        super().__init__(grid_in, grid_out, h)
        self.kd = kd

    def _count(self):
        return self._in.n if self.kd == Axis.x else self._in.nb * self._in.n

    def swapOffset(self, offset):
        o = _f32(offset)
        self._check(lib().vfps_kick_map_set_offset(self._h, _fptr(o), o.size))

    def getForce(self):
        out = np.empty(self._count(), np.float32)
        self._check(lib().vfps_kick_map_get_offset(self._h, _fptr(out),
                                                   out.size))
        return out


class DriftMap(KickMap):
    """DriftMap(in, out, slip, E0, it, interpol_clamp)."""

    def __init__(self, grid_in, grid_out, slip, E0, it, interpol_clamp,
                 oclh=None):
        s = _f32(slip)
        h = _new_map(lib().vfps_drift_map_create, grid_in, grid_out.handle,
                     _fptr(s), s.size, E0, it, int(interpol_clamp))
        super().__init__(grid_in, grid_out, it, interpol_clamp, Axis.x,
                         _handle=h)


class RFKickMap(KickMap):
    """RFKickMap(in, out, angle, f_RF, it, clamp) -- linear RF; use
    RFKickMap.sinusoidal(in, out, revolutionpart, V_RF, f_RF, V0, it,
    clamp) for the non-linear one."""

    def __init__(self, grid_in, grid_out, angle, f_RF, it, interpol_clamp,
                 oclh=None, _handle=None):
        h = _handle if _handle is not None else _new_map(
            lib().vfps_rf_kick_map_create_linear, grid_in, grid_out.handle,
            angle, f_RF, it, int(interpol_clamp))
        super().__init__(grid_in, grid_out, it, interpol_clamp, Axis.y,
                         _handle=h)

    @classmethod
    def sinusoidal(cls, grid_in, grid_out, revolutionpart, V_RF, f_RF, V0,
                   it, interpol_clamp):
        h = _new_map(lib().vfps_rf_kick_map_create, grid_in, grid_out.handle,
                     revolutionpart, V_RF, f_RF, V0, it, int(interpol_clamp))
        return cls(grid_in, grid_out, 0, 0, it, interpol_clamp, _handle=h)


class DynamicRFKickMap(KickMap):
    """DynamicRFKickMap(in, out, angle, revolutionpart, f_RF, phasespread,
    amplspread, modampl, modtimeincrement, steps, it, clamp) -- linear RF;
    DynamicRFKickMap.sinusoidal(in, out, revolutionpart, V_RF, f_RF, V0,
    ...) for the sinusoidal one.  ``seed`` keys the counter-based
    generator of the phase and amplitude noise."""

    def __init__(self, grid_in, grid_out, angle, revolutionpart, f_RF,
                 phasespread, amplspread, modampl, modtimeincrement, steps,
                 it, interpol_clamp, oclh=None, seed=0, _linear=True,
                 _v_rf=0.0, _v0=0.0):
        h = _new_map(lib().vfps_dynamic_rf_kick_map_create, grid_in,
                     grid_out.handle, int(_linear), angle, revolutionpart,
                     _v_rf, f_RF, _v0, phasespread, amplspread, modampl,
                     modtimeincrement, steps, it, int(interpol_clamp), seed)
        super().__init__(grid_in, grid_out, it, interpol_clamp, Axis.y,
                         _handle=h)

    @classmethod
    def sinusoidal(cls, grid_in, grid_out, revolutionpart, V_RF, f_RF, V0,
                   phasespread, amplspread, modampl, modtimeincrement, steps,
                   it, interpol_clamp, oclh=None, seed=0):
        return cls(grid_in, grid_out, 0.0, revolutionpart, f_RF,
                   phasespread, amplspread, modampl, modtimeincrement, steps,
                   it, interpol_clamp, oclh, seed, _linear=False,
                   _v_rf=V_RF, _v0=V0)

    def getPastModulation(self):
        """[(phase, amplitude)] of the applies so far (as logged)."""
        c = C.c_uint64()
        self._check(lib().vfps_dynamic_rf_get_modulation(self._h, None,
                                                         C.byref(c)))
        out = np.empty((c.value, 2), np.float32)
        if c.value:
            self._check(lib().vfps_dynamic_rf_get_modulation(
                self._h, _fptr(out), C.byref(c)))
        return out


class FokkerPlanckMap(SourceMap):
    """FokkerPlanckMap(in, out, xsize, ysize, fptype, fptrack, e1,
    derivation)."""

    def __init__(self, grid_in, grid_out, xsize, ysize, fptype, fptrack, e1,
                 dt, oclh=None):
        h = _new_map(lib().vfps_fokker_planck_map_create, grid_in,
                     grid_out.handle, xsize, ysize, fptype, fptrack, e1, dt)
        super().__init__(grid_in, grid_out, h)


class Identity(SourceMap):
    def __init__(self, grid_in, grid_out, oclh=None):
        h = _new_map(lib().vfps_identity_map_create, grid_in, grid_out.handle)
        super().__init__(grid_in, grid_out, h)


class WakePotentialMap(KickMap):
    """WakePotentialMap(in, out, field, it, interpol_clamp)."""

    def __init__(self, grid_in, grid_out, field, it, interpol_clamp,
                 oclh=None):
        h = _new_map(lib().vfps_wake_potential_map_create, grid_in,
                     grid_out.handle, field.handle, it, int(interpol_clamp))
        super().__init__(grid_in, grid_out, it, interpol_clamp, Axis.y,
                         _handle=h)
        self._field = field

    def update(self):
        self._check(lib().vfps_wake_map_update(self._h))


# ------------------------------------------------------------- impedances
class Impedance(_Handle):
    """Impedance(oclh, z, f_max) from a complex table, or
    Impedance.from_file(oclh, path, f_max)."""
    _destroy = "vfps_impedance_destroy"

    def __init__(self, oclh, z=None, f_max=1.0, _handle=None):
        self.ctx = oclh
        if _handle is not None:
            self._h = _handle
            return
        zz = np.ascontiguousarray(z, np.complex64)
        buf = zz.view(np.float32)
        h = C.c_void_p()
        check(lib().vfps_impedance_create(oclh.handle, _fptr(buf), zz.size,
                                          f_max, C.byref(h)), oclh.handle)
        self._h = h

    @classmethod
    def _wrap(cls, oclh, h):
        obj = cls.__new__(cls)
        obj.ctx = oclh
        obj._h = h
        return obj

    @classmethod
    def from_file(cls, oclh, path, f_max):
        h = C.c_void_p()
        check(lib().vfps_impedance_from_file(oclh.handle, path.encode(),
                                             f_max, C.byref(h)), oclh.handle)
        return Impedance._wrap(oclh, h)

    @property
    def handle(self):
        return self._h

    def nFreqs(self):
        n = C.c_size_t()
        self._check(lib().vfps_impedance_get(self._h, None, C.byref(n), None))
        return n.value

    def data(self):
        n = self.nFreqs()
        buf = np.empty(2 * n, np.float32)
        fm = C.c_double()
        self._check(lib().vfps_impedance_get(self._h, _fptr(buf), None,
                                             C.byref(fm)))
        return buf.view(np.complex64)

    def __getitem__(self, i):
        return self.data()[i]

    def fmax(self):
        fm = C.c_double()
        self._check(lib().vfps_impedance_get(self._h, None, None,
                                             C.byref(fm)))
        return fm.value

    def copy(self):
        h = C.c_void_p()
        self._check(lib().vfps_impedance_copy(self._h, C.byref(h)))
        return Impedance._wrap(self.ctx, h)

    def __iadd__(self, rhs):
        self._check(lib().vfps_impedance_add(self._h, rhs._h))
        return self

    def __add__(self, rhs):
        out = self.copy()
        out += rhs
        return out

    def swap(self, other):
        self._check(lib().vfps_impedance_swap(self._h, other._h))


def _model(fn, oclh, *args):
    h = C.c_void_p()
    check(fn(oclh.handle, *args, C.byref(h)), oclh.handle)
    return Impedance._wrap(oclh, h)


def FreeSpaceCSR(oclh, n, f_rev, f_max):
    return _model(lib().vfps_impedance_free_space_csr, oclh, n, f_rev, f_max)


def ParallelPlatesCSR(oclh, n, f0, f_max, g):
    return _model(lib().vfps_impedance_parallel_plates_csr, oclh, n, f0,
                  f_max, g)


def ResistiveWall(oclh, n, f0, f_max, L, s, xi, b):
    return _model(lib().vfps_impedance_resistive_wall, oclh, n, f0, f_max, L,
                  s, xi, b)


def ConstImpedance(oclh, n, f_max, Z):
    return _model(lib().vfps_impedance_const, oclh, n, f_max,
                  float(np.real(Z)), float(np.imag(Z)))


def CollimatorImpedance(oclh, n, f_max, outer, inner):
    return _model(lib().vfps_impedance_collimator, oclh, n, f_max, outer,
                  inner)


def makeImpedance(oclh, nfreqs, fmax, R_bend, frev, gap, use_csr=True, s=0.0,
                  xi=0.0, inner_coll_radius=0.0, impedance_file=""):
    """Returns None when no impedance contribution is selected."""
    h = C.c_void_p()
    check(lib().vfps_make_impedance(
        oclh.handle, nfreqs, fmax, R_bend, frev, gap, int(use_csr), s, xi,
        inner_coll_radius, impedance_file.encode() if impedance_file else None,
        C.byref(h)), oclh.handle)
    return Impedance._wrap(oclh, h) if h.value else None


# ----------------------------------------------------------- ElectricField
class ElectricField(_Handle):
    """ElectricField(ps, impedance, bucketnumbers, spacing_bins, oclh,
    f_rev, revolutionpart=1, wakescaling=0); ElectricField.wake(...) is the
    constructor taking Ib, E0, sigma_delta and dt."""
    _destroy = "vfps_field_destroy"

    def __init__(self, ps, impedance, bucketnumbers, spacing_bins, oclh=None,
                 f_rev=1.0, revolutionpart=1.0, wakescaling=0.0,
                 _handle=None):
        self.ctx = ps.ctx
        self._ps, self._imp = ps, impedance
        if _handle is not None:
            self._h = _handle
        else:
            bk = np.ascontiguousarray(bucketnumbers, np.uint32)
            h = C.c_void_p()
            self._check(lib().vfps_field_create(
                ps.handle, impedance.handle, bk.ctypes.data_as(_lib.U32P),
                spacing_bins, f_rev, revolutionpart, wakescaling, C.byref(h)))
            self._h = h

    @classmethod
    def wake(cls, ps, impedance, bucketnumbers, spacing_bins, oclh, f_rev,
             revolutionpart, Ib, E0, sigma_delta, dt):
        bk = np.ascontiguousarray(bucketnumbers, np.uint32)
        h = C.c_void_p()
        check(lib().vfps_field_create_wake(
            ps.handle, impedance.handle, bk.ctypes.data_as(_lib.U32P),
            spacing_bins, f_rev, revolutionpart, Ib, E0, sigma_delta, dt,
            C.byref(h)), ps.ctx.handle)
        return cls(ps, impedance, None, 0, _handle=h)

    @property
    def handle(self):
        return self._h

    def _info(self):
        ws, nm = C.c_float(), C.c_size_t()
        self._check(lib().vfps_field_info(self._h, C.byref(ws), C.byref(nm)))
        return ws.value, nm.value

    def getWakeScaling(self):
        return self._info()[0]

    def getNMax(self):
        return self._info()[1]

    def padBunchProfiles(self):
        self._check(lib().vfps_field_pad_bunch_profiles(self._h))

    def getPaddedBunchProfiles(self):
        out = np.empty(self.getNMax(), np.float32)
        self._check(lib().vfps_field_get_padded_profiles(self._h, _fptr(out)))
        return out

    def wakePotential(self):
        self._check(lib().vfps_field_wake_potential(self._h))
        return self.getWakePotentials()

    def getWakePotentials(self):
        out = np.empty((self._ps.nb, self._ps.n), np.float32)
        self._check(lib().vfps_field_get_wake_potential(self._h, _fptr(out)))
        return out

    def updateCSR(self, cutoff_frequency):
        self._check(lib().vfps_field_update_csr(self._h, cutoff_frequency))

    def getCSRSpectrum(self):
        out = np.empty((self._ps.nb, self.getNMax()), np.float32)
        self._check(lib().vfps_field_get_csr(self._h, _fptr(out), None, None))
        return out

    def getCSRPower(self):
        out = np.empty(self._ps.nb, np.float32)
        self._check(lib().vfps_field_get_csr(self._h, None, _fptr(out), None))
        return out

    @property
    def factor4Watts(self):
        f = C.c_double()
        self._check(lib().vfps_field_get_csr(self._h, None, None, C.byref(f)))
        return f.value


# ------------------------------------------------------------ batches
class BunchBatch(_Handle):
    """Many independent single-bunch simulations stepped by fused kernels
    (no reference counterpart)."""
    _destroy = "vfps_batch_destroy"

    def __init__(self, oclh, descs, impedances, data=None):
        self.ctx = oclh
        self.descs = list(descs)
        self._imps = list(impedances)
        arr = (BunchDesc * len(self.descs))(*self.descs)
        hs = (C.c_void_p * max(1, len(self._imps)))(
            *[z.handle for z in self._imps])
        d = None if data is None else _f32(data)
        h = C.c_void_p()
        check(lib().vfps_batch_create(oclh.handle, len(self.descs), arr, hs,
                                      len(self._imps),
                                      None if d is None else _fptr(d),
                                      C.byref(h)), oclh.handle)
        self._h = h
        self.cells = sum(int(x.n) ** 2 for x in self.descs)
        self.rows = sum(int(x.n) for x in self.descs)

    def layout(self, b):
        d, p = C.c_size_t(), C.c_size_t()
        self._check(lib().vfps_batch_layout(self._h, b, C.byref(d),
                                            C.byref(p)))
        return d.value, p.value

    def step(self, nsteps=1):
        self._check(lib().vfps_batch_step(self._h, nsteps))

    def run(self, density_in, nsteps, density_out=None, profiles_out=None,
            filling_out=None):
        fin = None if density_in is None else _fptr(density_in)
        self._check(lib().vfps_batch_run(
            self._h, fin, nsteps,
            None if density_out is None else _fptr(density_out),
            None if profiles_out is None else _fptr(profiles_out),
            None if filling_out is None else _fptr(filling_out)))

    def download(self):
        out = np.empty(self.cells, np.float32)
        self._check(lib().vfps_batch_download(self._h, _fptr(out)))
        return out

    def upload(self, data):
        d = _f32(data)
        self._check(lib().vfps_batch_upload(self._h, _fptr(d)))

    def density(self, b):
        full = self.download()
        off, _ = self.layout(b)
        n = int(self.descs[b].n)
        return full[off:off + n * n].reshape(n, n)

    def profiles(self):
        out = np.empty(self.rows, np.float32)
        self._check(lib().vfps_batch_get_profiles(self._h, _fptr(out)))
        return out

    def profile(self, b):
        _, off = self.layout(b)
        return self.profiles()[off:off + int(self.descs[b].n)]

    def set_beams(self, beam, bucket, spacing_bins, filling=None):
        """Couple bunches into multi-bunch beams: equal beam ids > 0 share
        one padded profile (bunch i at bucket[i] * spacing_bins); filling
        (optional) is each bunch's share of the charge."""
        nb = len(self.descs)
        be = np.ascontiguousarray(beam, np.uint32)
        bu = np.ascontiguousarray(bucket, np.uint32)
        if be.size != nb or bu.size != nb:
            raise InvalidArgument(
                1, "beam and bucket need one entry per bunch")
        fi = None
        if filling is not None:
            fi = np.ascontiguousarray(filling, np.float32)
            if fi.size != nb:
                raise InvalidArgument(1, "filling needs one entry per bunch")
        self._check(lib().vfps_batch_set_beams(
            self._h, be.ctypes.data_as(_lib.U32P),
            bu.ctypes.data_as(_lib.U32P), int(spacing_bins),
            None if fi is None else _fptr(fi)))

    def set_csr(self, impedances, impedance, fc, freq_scale, every=1,
                capacity=64):
        """Record every bunch's CSR power (the reference's updateCSR) at
        steps with step % every == 0 into a ring of `capacity` slots.
        impedances: Impedance objects; impedance, fc, freq_scale: per bunch
        (impedance -1: no CSR for that bunch); every=0 switches it off."""
        nb = len(self.descs)
        self._csr_imps = list(impedances)
        hs = (C.c_void_p * max(1, len(self._csr_imps)))(
            *[z.handle for z in self._csr_imps])
        idx = np.ascontiguousarray(impedance, np.int32)
        f = np.ascontiguousarray(fc, np.float64)
        sc = np.ascontiguousarray(freq_scale, np.float64)
        if idx.size != nb or f.size != nb or sc.size != nb:
            raise InvalidArgument(
                1, "impedance, fc and freq_scale need one entry per bunch")
        self._check(lib().vfps_batch_set_csr(
            self._h, hs, len(self._csr_imps), idx.ctypes.data_as(_lib.I32P),
            f.ctypes.data_as(_lib.DP), sc.ctypes.data_as(_lib.DP),
            int(every), int(capacity)))
        self._csr_cap = int(capacity) if every else 0

    def csr(self):
        """(steps, power[len(steps)][nb]) of the recorded steps in order."""
        nb = len(self.descs)
        cap = getattr(self, "_csr_cap", 0)
        if cap == 0:
            raise InvalidArgument(1, "CSR recording is off")
        power = np.empty((cap, nb), np.float32)
        steps = np.empty(cap, np.uint64)
        self._check(lib().vfps_batch_get_csr(
            self._h, _fptr(power), steps.ctypes.data_as(_lib.U64P)))
        ok = steps != np.uint64(0xffffffffffffffff)
        order = np.argsort(steps[ok], kind="stable")
        return steps[ok][order].astype(np.int64), power[ok][order]

    def potential_well(self, iterations=200, mix=0.5):
        """Replace every density by the stationary state of its step below
        threshold (the Haissinski potential well written in the invariant
        of the discrete step: kick-drift, or rotation and wake kick; the
        members of a coupled beam together); returns the last relative
        change of each profile in the fixed-point iteration."""
        out = np.zeros(len(self.descs), np.float32)
        self._check(lib().vfps_batch_potential_well(
            self._h, int(iterations), float(mix), _fptr(out)))
        return out

    def wake(self):
        out = np.empty(self.rows, np.float32)
        self._check(lib().vfps_batch_get_wake(self._h, _fptr(out)))
        return out

    def filling(self):
        out = np.empty(len(self.descs), np.float64)
        self._check(lib().vfps_batch_get_filling(
            self._h, out.ctypes.data_as(_lib.DP)))
        return out

    def info(self):
        launches, rows = C.c_uint32(), C.c_uint32()
        self._check(lib().vfps_batch_info(self._h, C.byref(launches),
                                          C.byref(rows)))
        return launches.value, rows.value

    KERNELS = ("k_bmaps0f", "k_bmaps0", "k_bmaps0<4>", "k_bmaps0w",
               "k_bmaps1")

    def kernel_tiles(self):
        """Tiles each maps kernel of the step walks, by kernel name."""
        t = (C.c_uint32 * len(self.KERNELS))()
        self._check(lib().vfps_batch_kernel_tiles(self._h, t,
                                                  len(self.KERNELS)))
        return dict(zip(self.KERNELS, list(t)))

    def set_wake_mode(self, mode):
        """0: wake potentials on the CUDA cores (default); 1: on the tensor
        cores (TF32 split products, FP32 accumulation)."""
        self._check(lib().vfps_batch_set_wake_mode(self._h, int(mode)))

    def kernel_times(self, nsteps=20):
        """Advance nsteps steps kernel by kernel; mean ms per step of the
        wake, chain-0 and chain-1 kernels (CUDA events on the library's
        stream)."""
        ms = (C.c_float * 3)()
        self._check(lib().vfps_batch_kernel_times(self._h, nsteps, ms))
        return {"wake": ms[0], "k_bmaps0": ms[1], "k_bmaps1": ms[2]}
