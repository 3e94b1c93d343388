"""Loader and ctypes signatures of libvfps.so.

The library must have been built (``inovesa_gb300.build.build()``); there
is no CPU fallback.  Loading fails with an ImportError naming the missing
file, and every call that returns a non-zero status raises VfpsError.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libvfps.so")

VFPS_OK = 0
VFPS_ERR_INVALID_ARGUMENT = 1
VFPS_ERR_CUDA = 2
VFPS_ERR_OUT_OF_MEMORY = 3
VFPS_ERR_NUMERIC = 4
VFPS_ERR_TIMEOUT = 5
VFPS_ERR_IO = 6


class VfpsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("vfps error %d: %s" % (code, msg))
        self.code = code


class InvalidArgument(VfpsError, ValueError):
    """std::invalid_argument of the reference."""


class BunchDesc(C.Structure):
    """Mirror of vfps_bunch_desc (include/vfps.h)."""
    _fields_ = [
        ("n", C.c_uint32), ("chain", C.c_int32), ("it", C.c_int32),
        ("clamp", C.c_int32), ("axes", C.c_double * 6), ("zoom", C.c_double),
        ("angle", C.c_double), ("rf_linear", C.c_int32),
        ("rf_angle", C.c_double), ("rf_revpart", C.c_double),
        ("rf_vrf", C.c_double), ("rf_v0", C.c_double),
        ("rf_bl2phase", C.c_double), ("rf_phase", C.c_double),
        ("slip", C.c_double * 3), ("nslip", C.c_int32), ("e0", C.c_double),
        ("e1", C.c_double), ("fptype", C.c_int32), ("derivation", C.c_int32),
        ("wakescaling", C.c_double), ("renormalize", C.c_int32),
        ("impedance", C.c_int32),
    ]


class WsNet(C.Structure):
    """Mirror of vfps_ws_net (include/vfps.h)."""
    _fields_ = [("nin", C.c_uint32), ("nh", C.c_uint32),
                ("nlat", C.c_uint32), ("npix", C.c_uint32),
                ("w1", C.c_void_p), ("b1", C.c_void_p),
                ("w2", C.c_void_p), ("b2", C.c_void_p),
                ("w3", C.c_void_p), ("b3", C.c_void_p),
                ("wd", C.c_void_p), ("bd", C.c_void_p)]


_lib = None
P = C.c_void_p
PP = C.POINTER(C.c_void_p)
FP = C.POINTER(C.c_float)
DP = C.POINTER(C.c_double)
U32P = C.POINTER(C.c_uint32)
SZP = C.POINTER(C.c_size_t)
I32P = C.POINTER(C.c_int32)
U64P = C.POINTER(C.c_uint64)
i32, u32, u64, sz, dbl, flt = (C.c_int, C.c_uint32, C.c_uint64, C.c_size_t,
                               C.c_double, C.c_float)

SIGNATURES = {
    "vfps_create": [PP, i32],
    "vfps_destroy": [P],
    "vfps_last_error": [P],
    "vfps_synchronize": [P],
    "vfps_stream": [P],
    "vfps_device_status": [P, C.POINTER(C.c_int)],
    "vfps_host_alloc": [P, sz, PP],
    "vfps_host_free": [P, P],
    "vfps_selftest_wait_timeout": [P, C.c_uint64],
    "vfps_ps_create": [P, u32, u32, DP, dbl, dbl, FP, dbl, FP, PP],
    "vfps_ps_copy": [P, PP],
    "vfps_ps_destroy": [P],
    "vfps_ps_swap": [P, P],
    "vfps_ps_assign": [P, P],
    "vfps_ps_download": [P, FP],
    "vfps_ps_upload": [P, FP],
    "vfps_ps_device_data": [P],
    "vfps_ps_shape": [P, U32P, U32P],
    "vfps_ps_axis": [P, i32, FP, FP, FP],
    "vfps_ps_update_x_projection": [P],
    "vfps_ps_update_y_projection": [P],
    "vfps_ps_integrate": [P],
    "vfps_ps_normalize": [P],
    "vfps_ps_integrate_and_normalize": [P],
    "vfps_ps_variance": [P, i32],
    "vfps_ps_get_projection": [P, i32, FP],
    "vfps_ps_set_projection": [P, i32, u32, FP],
    "vfps_ps_get_filling": [P, FP, DP],
    "vfps_ps_get_moments": [P, i32, FP, FP, FP],
    "vfps_rotation_map_create": [P, P, u32, u32, flt, i32, i32, u32, PP],
    "vfps_kick_map_create": [P, P, i32, i32, i32, PP],
    "vfps_kick_map_set_offset": [P, FP, sz],
    "vfps_kick_map_get_offset": [P, FP, sz],
    "vfps_drift_map_create": [P, P, FP, u32, flt, i32, i32, PP],
    "vfps_rf_kick_map_create_linear": [P, P, flt, flt, i32, i32, PP],
    "vfps_rf_kick_map_create": [P, P, flt, flt, flt, flt, i32, i32, PP],
    "vfps_dynamic_rf_kick_map_create": [P, P, i32, flt, flt, flt, flt, flt,
                                        flt, flt, flt, dbl, u32, i32, i32,
                                        u32, PP],
    "vfps_dynamic_rf_get_modulation": [P, FP, C.POINTER(C.c_uint64)],
    "vfps_philox4x32": [U32P, U32P, U32P],
    "vfps_fokker_planck_map_create": [P, P, u32, u32, i32, i32, flt, i32, PP],
    "vfps_identity_map_create": [P, P, PP],
    "vfps_wake_potential_map_create": [P, P, P, i32, i32, PP],
    "vfps_wake_map_update": [P],
    "vfps_map_apply": [P],
    "vfps_map_apply_to": [P, FP, sz],
    "vfps_map_destroy": [P],
    "vfps_impedance_create": [P, FP, sz, dbl, PP],
    "vfps_impedance_free_space_csr": [P, sz, flt, flt, PP],
    "vfps_impedance_parallel_plates_csr": [P, sz, flt, flt, dbl, PP],
    "vfps_impedance_resistive_wall": [P, sz, flt, flt, dbl, dbl, dbl, dbl,
                                      PP],
    "vfps_impedance_const": [P, sz, flt, flt, flt, PP],
    "vfps_impedance_collimator": [P, sz, flt, dbl, dbl, PP],
    "vfps_impedance_from_file": [P, C.c_char_p, dbl, PP],
    "vfps_make_impedance": [P, sz, flt, dbl, dbl, dbl, i32, dbl, dbl, dbl,
                            C.c_char_p, PP],
    "vfps_impedance_add": [P, P],
    "vfps_impedance_copy": [P, PP],
    "vfps_impedance_swap": [P, P],
    "vfps_impedance_get": [P, FP, SZP, DP],
    "vfps_impedance_destroy": [P],
    "vfps_field_create": [P, P, U32P, u32, dbl, dbl, dbl, PP],
    "vfps_field_create_wake": [P, P, U32P, u32, dbl, dbl, dbl, dbl, dbl, dbl,
                               PP],
    "vfps_field_pad_bunch_profiles": [P],
    "vfps_field_get_padded_profiles": [P, FP],
    "vfps_field_wake_potential": [P],
    "vfps_field_get_wake_potential": [P, FP],
    "vfps_field_info": [P, FP, SZP],
    "vfps_field_update_csr": [P, flt],
    "vfps_field_get_csr": [P, FP, FP, DP],
    "vfps_field_destroy": [P],
    "vfps_batch_create": [P, u32, C.POINTER(BunchDesc), PP, u32, FP, PP],
    "vfps_batch_step": [P, u64],
    "vfps_batch_run": [P, FP, u64, FP, FP, FP],
    "vfps_batch_layout": [P, u32, SZP, SZP],
    "vfps_batch_download": [P, FP],
    "vfps_batch_upload": [P, FP],
    "vfps_batch_get_profiles": [P, FP],
    "vfps_batch_get_filling": [P, DP],
    "vfps_batch_get_wake": [P, FP],
    "vfps_batch_potential_well": [P, C.c_uint32, C.c_float, FP],
    "vfps_batch_set_beams": [P, U32P, U32P, C.c_uint32, FP],
    "vfps_batch_set_csr": [P, PP, C.c_uint32, I32P, DP, DP, C.c_uint32,
                           C.c_uint32],
    "vfps_batch_get_csr": [P, FP, U64P],
    "vfps_batch_info": [P, U32P, U32P],
    "vfps_batch_kernel_tiles": [P, U32P, u32],
    "vfps_batch_kernel_times": [P, u32, FP],
    "vfps_charge_noalloc": [P, P, u32, u32, flt, DP],
    "vfps_batch_set_wake_mode": [P, i32],
    "vfps_ws_forward": [P, C.POINTER(WsNet), P, u32, P, P, P, P, P, P, P,
                        u32],
    "vfps_ws_backward": [P, C.POINTER(WsNet), C.POINTER(WsNet), P, u32, P,
                         P, P, P, P, P, P],
    "vfps_ws_adam": [P, P, P, P, P, P, sz, flt, flt, flt, flt, u32],
    "vfps_batch_destroy": [P],
}

RESTYPES = {
    "vfps_last_error": C.c_char_p,
    "vfps_stream": C.c_void_p,
    "vfps_ps_device_data": C.c_void_p,
}


def lib():
    """Load libvfps.so (built in-tree) and declare its signatures."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libvfps.so is not built (%s); run "
                              "inovesa_gb300.build.build() first" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = RESTYPES.get(name, C.c_int)
        _lib = L
    return _lib


def check(rc, ctx=None):
    """Raise for a non-zero status, with the context's last message."""
    if rc == VFPS_OK:
        return
    msg = lib().vfps_last_error(ctx)
    msg = msg.decode() if msg else ""
    if rc == VFPS_ERR_INVALID_ARGUMENT:
        raise InvalidArgument(rc, msg)
    raise VfpsError(rc, msg)
