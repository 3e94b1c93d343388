"""ctypes binding of the oracle (test infrastructure only).

The oracle is the checker: tests/, the smoke test and bench.py's CPU
baseline leg use it to judge or time the reference algorithm on the CPU.
Nothing in the product package imports this module.

Every function takes a ``dtype`` argument: ``np.float32`` runs the float
restatement of the reference CPU build, ``np.float64`` the FP64 oracle.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        _declare(_lib)
    return _lib


class BunchDesc(C.Structure):
    """Mirror of ``oracle_bunch_desc`` in vfps_oracle.cpp."""
    _fields_ = [
        ("n", C.c_int), ("chain", C.c_int), ("it", C.c_int),
        ("clamp", C.c_int),
        ("qmin", C.c_double), ("qmax", C.c_double), ("qscale", C.c_double),
        ("pmin", C.c_double), ("pmax", C.c_double), ("pscale", C.c_double),
        ("zoom", C.c_double), ("angle", C.c_double),
        ("rf_linear", C.c_int), ("rf_angle", C.c_double),
        ("rf_revpart", C.c_double), ("rf_vrf", C.c_double),
        ("rf_v0", C.c_double), ("rf_bl2phase", C.c_double),
        ("rf_phase", C.c_double),
        ("slip", C.c_double * 3), ("nslip", C.c_int), ("e0", C.c_double),
        ("e1", C.c_double), ("fptype", C.c_int), ("derivation", C.c_int),
        ("wakescaling", C.c_double), ("renormalize", C.c_int),
    ]


_P = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_DP = C.POINTER(C.c_double)


def _declare(L):
    def sig(name, res, args):
        for suf in ("_f32", "_f64"):
            f = getattr(L, name + suf, None)
            if f is not None:
                f.restype = res
                f.argtypes = args
    u32, i, d, sz = C.c_uint32, C.c_int, C.c_double, C.c_size_t
    sig("oracle_ruler", None, [u32, d, d, _P, _P, _P])
    sig("oracle_simpson", None, [u32, d, d, _P])
    sig("oracle_ps_init", i, [u32, u32, _DP, _P, d, _P, _P, _P, _P, _P, _P])
    sig("oracle_project_x", None, [u32, u32, _P, _P, _P])
    sig("oracle_project_y", None, [u32, u32, _P, _P, _P])
    sig("oracle_integrate", None, [u32, u32, _P, _P, _P, _P])
    sig("oracle_normalize", None, [u32, u32, _P, _P, _P])
    sig("oracle_moments", None, [u32, u32, _P, d, _P, _P, _P, _P, _P])
    sig("oracle_rotation", i, [u32, u32, _DP, d, i, i, C.c_long, _P, _P])
    sig("oracle_rotation_particle", None, [u32, _DP, d, _P])
    sig("oracle_kick_stencils", None, [u32, i, _P, sz, _U32P, _P])
    sig("oracle_kick_apply", None, [i, u32, u32, i, _U32P, _P, _P, _P])
    sig("oracle_kick_particle", None, [i, u32, _P, _P])
    sig("oracle_drift_offsets", None, [u32, _DP, _DP, i, d, _P])
    sig("oracle_rf_offsets", None, [u32, _DP, i, d, d, d, d, d, d, d, _P])
    sig("oracle_fp_stencils", i, [u32, _DP, d, i, i, _U32P, _P])
    sig("oracle_fp_apply", None, [u32, u32, i, _U32P, _P, _P, _P])
    sig("oracle_wake_potential", None,
        [u32, u32, sz, _P, _U32P, sz, _P, d, _P, _P])
    sig("oracle_csr", None, [u32, sz, _P, _P, d, d, d, _P, _P])
    sig("oracle_sim_create", _P, [i, C.POINTER(BunchDesc), _P, sz, _P])
    sig("oracle_sim_step", None, [_P, C.c_long, i])
    sig("oracle_sim_get", None, [_P, i, i, _P])
    sig("oracle_sim_destroy", None, [_P])
    L.oracle_airy.restype = None
    L.oracle_airy.argtypes = [d, _DP, C.POINTER(i)]
    L.oracle_z_free_space.argtypes = [sz, C.c_float, C.c_float, _P]
    L.oracle_z_parallel_plates.argtypes = [sz, C.c_float, C.c_float, d, _P]
    L.oracle_z_resistive_wall.argtypes = [sz, C.c_float, C.c_float, d, d, d,
                                          d, _P]
    L.oracle_z_const.argtypes = [sz, C.c_float, C.c_float, _P]
    L.oracle_z_collimator.argtypes = [sz, d, d, _P]
    L.oracle_make_impedance.restype = i
    L.oracle_make_impedance.argtypes = [sz, C.c_float, d, d, d, i, d, d, d,
                                        _P]
    L.oracle_rfft_f64.argtypes = [_P, sz, _P]


def _suffix(dtype):
    return "_f32" if np.dtype(dtype) == np.float32 else "_f64"


def _fn(name, dtype):
    return getattr(lib(), name + _suffix(dtype))


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _ax6(axes):
    return (C.c_double * 6)(*[float(v) for v in axes])


def _arr(x, dtype):
    return np.ascontiguousarray(x, dtype=dtype)


# ---------------------------------------------------------------- ruler / PS
def ruler(n, mn, mx, dtype=np.float64):
    v = np.zeros(n, dtype)
    d = np.zeros(1, dtype)
    z = np.zeros(1, dtype)
    _fn("oracle_ruler", dtype)(n, mn, mx, _ptr(v), _ptr(d), _ptr(z))
    return v, d[0], z[0]


def simpson(n, mn, mx, dtype=np.float64):
    ws = np.zeros(n, dtype)
    _fn("oracle_simpson", dtype)(n, mn, mx, _ptr(ws))
    return ws


def ps_init(n, axes, filling=(1.0,), zoom=1.0, data=None, dtype=np.float64):
    """PhaseSpace constructor. axes = (qmin, qmax, qscale, pmin, pmax,
    pscale). Raises ValueError for an unnormalised filling."""
    fs = _arr(filling, dtype)
    nb = fs.size
    out = np.zeros((nb, n, n), dtype)
    px = np.zeros((nb, n), dtype)
    py = np.zeros((nb, n), dtype)
    fill = np.zeros(nb, dtype)
    integ = np.zeros(1, dtype)
    d = None if data is None else _arr(data, dtype)
    rc = _fn("oracle_ps_init", dtype)(
        nb, n, _ax6(axes), _ptr(fs), zoom,
        None if d is None else _ptr(d), _ptr(out), _ptr(px), _ptr(py),
        _ptr(fill), _ptr(integ))
    if rc != 0:
        raise ValueError('Argument "filling" not normalized.')
    return dict(data=out, projx=px, projy=py, filling=fill,
                integral=integ[0])


def project_x(data, ws, dtype=np.float64):
    data = _arr(data, dtype)
    nb, n = data.shape[0], data.shape[1]
    out = np.zeros((nb, n), dtype)
    _fn("oracle_project_x", dtype)(nb, n, _ptr(data), _ptr(_arr(ws, dtype)),
                                   _ptr(out))
    return out


def project_y(data, ws, dtype=np.float64):
    data = _arr(data, dtype)
    nb, n = data.shape[0], data.shape[1]
    out = np.zeros((nb, n), dtype)
    _fn("oracle_project_y", dtype)(nb, n, _ptr(data), _ptr(_arr(ws, dtype)),
                                   _ptr(out))
    return out


def integrate(proj, ws, dtype=np.float64):
    proj = _arr(proj, dtype)
    nb, n = proj.shape
    fill = np.zeros(nb, dtype)
    tot = np.zeros(1, dtype)
    _fn("oracle_integrate", dtype)(nb, n, _ptr(proj), _ptr(_arr(ws, dtype)),
                                   _ptr(fill), _ptr(tot))
    return fill, tot[0]


def normalize(data, filling_set, filling, dtype=np.float64):
    data = np.array(data, dtype=dtype, copy=True)
    nb, n = data.shape[0], data.shape[1]
    _fn("oracle_normalize", dtype)(nb, n, _ptr(data),
                                   _ptr(_arr(filling_set, dtype)),
                                   _ptr(_arr(filling, dtype)))
    return data


def moments(axis_values, delta, proj, filling_set, filling,
            dtype=np.float64):
    proj = _arr(proj, dtype)
    nb, n = proj.shape
    avg = np.zeros(nb, dtype)
    var = np.zeros(nb, dtype)
    _fn("oracle_moments", dtype)(nb, n, _ptr(_arr(axis_values, dtype)),
                                 float(delta), _ptr(proj),
                                 _ptr(_arr(filling_set, dtype)),
                                 _ptr(_arr(filling, dtype)), _ptr(avg),
                                 _ptr(var))
    return avg, var


# ------------------------------------------------------------------- maps
def rotation(data, axes, angle, it, clamp=False, rotmapsize=None,
             dtype=np.float64):
    data = _arr(data, dtype)
    if data.ndim == 2:
        data = data[None]
    nb, n = data.shape[0], data.shape[1]
    if rotmapsize is None:
        rotmapsize = n * n if clamp else 0
    out = np.zeros_like(data)
    rc = _fn("oracle_rotation", dtype)(nb, n, _ax6(axes), float(angle), it,
                                       int(clamp), rotmapsize, _ptr(data),
                                       _ptr(out))
    if rc != 0:
        raise ValueError("Clamping only supported with cubic interpolation "
                         "and rotmapsize > 0.")
    return out


def rotation_particle(n, axes, angle, pos, dtype=np.float64):
    p = _arr(pos, dtype).copy()
    _fn("oracle_rotation_particle", dtype)(n, _ax6(axes), float(angle),
                                           _ptr(p))
    return p


def kick_stencils(kd, it, offset, dtype=np.float64):
    off = _arr(offset, dtype)
    idx = np.zeros(off.size * it, np.uint32)
    w = np.zeros(off.size * it, dtype)
    _fn("oracle_kick_stencils", dtype)(
        kd, it, _ptr(off), off.size, idx.ctypes.data_as(_U32P), _ptr(w))
    return idx, w


def kick_apply(axis, data, it, idx, w, dtype=np.float64):
    data = _arr(data, dtype)
    if data.ndim == 2:
        data = data[None]
    nb, n = data.shape[0], data.shape[1]
    out = np.zeros_like(data)
    idx = np.ascontiguousarray(idx, np.uint32)
    _fn("oracle_kick_apply", dtype)(axis, nb, n, it, idx.ctypes.data_as(_U32P),
                                    _ptr(_arr(w, dtype)), _ptr(data),
                                    _ptr(out))
    return out


def kick(axis, data, it, offset, dtype=np.float64):
    """KickMap with swapOffset(offset) then apply()."""
    data = _arr(data, dtype)
    n = data.shape[-1]
    idx, w = kick_stencils(n, it, offset, dtype)
    return kick_apply(axis, data, it, idx, w, dtype)


def kick_particle(axis, n, offset, pos, dtype=np.float64):
    p = _arr(pos, dtype).copy()
    _fn("oracle_kick_particle", dtype)(axis, n, _ptr(_arr(offset, dtype)),
                                       _ptr(p))
    return p


def drift_offsets(n, axes, slip, e0, dtype=np.float64):
    off = np.zeros(n, dtype)
    s = (C.c_double * 3)(*(list(slip) + [0.0] * (3 - len(slip))))
    _fn("oracle_drift_offsets", dtype)(n, _ax6(axes), s, len(slip), e0,
                                       _ptr(off))
    return off


def rf_offsets(n, axes, linear, angle=0.0, revpart=0.0, vrf=0.0, v0=0.0,
               bl2phase=1.0, phase=0.0, ampl=1.0, dtype=np.float64):
    off = np.zeros(n, dtype)
    _fn("oracle_rf_offsets", dtype)(n, _ax6(axes), int(linear), angle,
                                    revpart, vrf, v0, bl2phase, phase, ampl,
                                    _ptr(off))
    return off


def fp_stencils(n, axes, e1, fptype=3, derivation=4, dtype=np.float64):
    idx = np.zeros(n * derivation, np.uint32)
    w = np.zeros(n * derivation, dtype)
    rc = _fn("oracle_fp_stencils", dtype)(n, _ax6(axes), e1, fptype,
                                          derivation,
                                          idx.ctypes.data_as(_U32P), _ptr(w))
    if rc != 0:
        raise ValueError("derivation must be 3 or 4")
    return idx, w


def fp_apply(data, derivation, idx, w, dtype=np.float64):
    data = _arr(data, dtype)
    if data.ndim == 2:
        data = data[None]
    nb, n = data.shape[0], data.shape[1]
    out = np.zeros_like(data)
    idx = np.ascontiguousarray(idx, np.uint32)
    _fn("oracle_fp_apply", dtype)(nb, n, derivation, idx.ctypes.data_as(_U32P),
                                  _ptr(_arr(w, dtype)), _ptr(data), _ptr(out))
    return out



def fp_particle(mode, n, derivation, idx, w, pos, density=None, e1=0.0,
                dp=1.0, noise=None):
    """FokkerPlanckMap::applyTo (src/SM/FokkerPlanckMap.cpp:214-268) for
    particles pos[k] = (x, y) in mesh units, in float arithmetic as the
    reference (interpol_t = meshdata_t = float).  Small cases only (a
    Python loop per particle).

    mode 1 (approximation1): the stencil's mean index displacement at
      yi = floor(y): y += sum_j (yi - idx_j) w_j, clamped to [1, n-1].
      The reference bounds yi by n (one row past the table); here yi is
      bounded by n - 1, which only matters for y >= n - 1.
    mode 2 (approximation2): the same displacement weighted by the
      density of bunch 0 at row xi = floor(x): offset = sum_j v_j (idx_j -
      yi) / sum_j v_j with v_j = f[xi][idx_j] w_j; y += offset, clamped.
      Particles below the mesh (xi or yi < 0) are left where they are (the
      reference indexes before the mesh there).
    mode 3 (stochastic): y -= y e1 + noise[k], the noise drawn from
      N(0, sqrt(2 e1)/dp) by the caller (the reference draws it from an
      unseeded generator)."""
    f32 = np.float32
    p = np.array(pos, np.float32).reshape(-1, 2).copy()
    idx = np.asarray(idx, np.uint32).reshape(n, derivation)
    w = np.asarray(w, np.float32).reshape(n, derivation)
    lo, hi = f32(1), f32(n - 1)
    for k in range(p.shape[0]):
        y = p[k, 1]
        if mode == 1:
            yi = min(max(int(np.floor(y)), 0), n - 1)
            off = f32(0)
            for j in range(derivation):
                dy = f32(yi) - f32(idx[yi, j])
                off = f32(off + f32(dy * w[yi, j]))
            p[k, 1] = max(lo, min(f32(y + off), hi))
        elif mode == 2:
            xi = min(int(np.floor(p[k, 0])), n - 1)
            yi = min(int(np.floor(y)), n - 1)
            if xi < 0 or yi < 0:
                continue
            d = np.asarray(density, np.float32).reshape(-1, n, n)[0]
            off = f32(0)
            charge = f32(0)
            for j in range(derivation):
                h = int(idx[yi, j])
                v = f32(d[xi, h] * w[yi, j])
                charge = f32(charge + v)
                off = f32(off + f32(v * f32(h - yi)))
            with np.errstate(divide="ignore", invalid="ignore"):
                # no charge under the stencil: NaN, which the clamp below
                # turns into 1 as std::min/std::max do in the reference
                off = f32(off / charge)
            p[k, 1] = max(lo, min(f32(y + off), hi))
        elif mode == 3:
            p[k, 1] = f32(y - f32(f32(y * f32(e1)) + f32(noise[k])))
    return p

# -------------------------------------------------------------- impedance
def airy(x):
    out = (C.c_double * 4)()
    ovf = C.c_int(0)
    lib().oracle_airy(float(x), out, C.byref(ovf))
    return tuple(out), bool(ovf.value)


def _z(n):
    return np.zeros(2 * n, np.float32)


def _zc(buf):
    return buf.view(np.complex64)


def z_free_space(n, f_rev, f_max):
    b = _z(n)
    lib().oracle_z_free_space(n, f_rev, f_max, _ptr(b))
    return _zc(b)


def z_parallel_plates(n, f0, f_max, g):
    b = _z(n)
    lib().oracle_z_parallel_plates(n, f0, f_max, g, _ptr(b))
    return _zc(b)


def z_resistive_wall(n, f0, f_max, L, s, xi, radius):
    b = _z(n)
    lib().oracle_z_resistive_wall(n, f0, f_max, L, s, xi, radius, _ptr(b))
    return _zc(b)


def z_const(n, z):
    b = _z(n)
    lib().oracle_z_const(n, float(np.real(z)), float(np.imag(z)), _ptr(b))
    return _zc(b)


def z_collimator(n, outer, inner):
    b = _z(n)
    lib().oracle_z_collimator(n, outer, inner, _ptr(b))
    return _zc(b)


def make_impedance(nfreqs, fmax, r_bend, frev, gap, use_csr=True, s=0.0,
                   xi=0.0, coll=0.0):
    b = _z(nfreqs)
    rc = lib().oracle_make_impedance(nfreqs, fmax, r_bend, frev, gap,
                                     int(use_csr), s, xi, coll, _ptr(b))
    return None if rc else _zc(b)


# ---------------------------------------------------------- electric field
def wake_potential(proj, Z, wakescaling, buckets=None, spacing=0,
                   dtype=np.float64, return_padded=False):
    proj = _arr(proj, dtype)
    if proj.ndim == 1:
        proj = proj[None]
    nb, n = proj.shape
    Z = np.ascontiguousarray(Z, np.complex64)
    nmax = Z.size
    bk = np.ascontiguousarray(
        np.zeros(nb) if buckets is None else buckets, np.uint32)
    # the padded profile holds every bunch at bucket * spacing
    # (src/PS/ElectricField.cpp:255-263)
    if int(bk.max()) * int(spacing) + n > nmax:
        raise ValueError("bunches do not fit in the padded profile")
    wake = np.zeros((nb, n), dtype)
    pad = np.zeros(nmax, dtype)
    _fn("oracle_wake_potential", dtype)(
        nb, n, nmax, _ptr(proj), bk.ctypes.data_as(_U32P), spacing, _ptr(Z),
        float(wakescaling), _ptr(wake), _ptr(pad))
    return (wake, pad) if return_padded else wake


def csr(proj, Z, dq, fc, freq_scale, dtype=np.float64):
    proj = _arr(proj, dtype)
    n = proj.size
    Z = np.ascontiguousarray(Z, np.complex64)
    nmax = Z.size
    spec = np.zeros(nmax, dtype)
    power = np.zeros(1, dtype)
    _fn("oracle_csr", dtype)(n, nmax, _ptr(proj), _ptr(Z), float(dq),
                             float(fc), float(freq_scale), _ptr(spec),
                             _ptr(power))
    return spec, power[0]


def rfft(x):
    x = _arr(x, np.float64)
    out = np.zeros(2 * x.size, np.float64)
    lib().oracle_rfft_f64(_ptr(x), x.size, _ptr(out))
    return out.view(np.complex128)


# ------------------------------------------------------------- solver loop
class Sim:
    """Independent bunches stepped like the reference solver loop."""

    def __init__(self, descs, Z=None, data=None, dtype=np.float64):
        self.dtype = np.dtype(dtype)
        arr = (BunchDesc * len(descs))(*descs)
        self.descs = list(descs)
        self._Z = None if Z is None else np.ascontiguousarray(Z, np.complex64)
        nmax = 0 if self._Z is None else self._Z.size
        d = None if data is None else _arr(data, dtype)
        self._h = _fn("oracle_sim_create", dtype)(
            len(descs), arr, None if d is None else _ptr(d), nmax,
            None if self._Z is None else _ptr(self._Z))

    def step(self, nsteps=1, threads=1):
        _fn("oracle_sim_step", self.dtype)(self._h, nsteps, threads)

    def _get(self, b, what, size):
        out = np.zeros(size, self.dtype)
        _fn("oracle_sim_get", self.dtype)(self._h, b, what, _ptr(out))
        return out

    def density(self, b):
        n = self.descs[b].n
        return self._get(b, 0, n * n).reshape(n, n)

    def profile(self, b):
        return self._get(b, 1, self.descs[b].n)

    def wake(self, b):
        return self._get(b, 2, self.descs[b].n)

    def filling(self, b):
        return self._get(b, 3, 1)[0]

    def close(self):
        if self._h:
            _fn("oracle_sim_destroy", self.dtype)(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
