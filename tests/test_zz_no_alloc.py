"""vfps_charge_noalloc (charge integrals from raw device pointers, no
allocation) against the PhaseSpace path that owns its buffers
(vfps_ps_update_x_projection + vfps_ps_integrate).

Collected last (file name) so that it also runs after every other GPU
test in the same process; it passes alone in a fresh process too.
Tolerance: both paths add in the same order, so the FP64 integrals agree
to 1e-12 relative; the PhaseSpace path hands per-bunch values out as
float, compared at 1e-6 relative.
"""
import ctypes as C

import numpy as np
import pytest

from inovesa_gb300 import _lib
from inovesa_gb300 import vfps as V

pytestmark = pytest.mark.gpu


def noalloc(ctx, ptr, nb, n, delta):
    out = np.full(nb, np.nan, np.float64)
    rc = _lib.lib().vfps_charge_noalloc(
        ctx.handle, ptr, nb, n, delta,
        out.ctypes.data_as(C.POINTER(C.c_double)))
    return rc, out


def test_charge_noalloc_matches_phase_space(gpu_ctx):
    nb, n = 3, 192
    rng = np.random.default_rng(7)
    data = rng.random((nb, n, n), dtype=np.float32)
    ps = V.PhaseSpace(-6.0, 6.0, 1.0, -6.0, 6.0, 1.0, gpu_ctx,
                      filling=(0.5, 0.3, 0.2), data=data, n=n)
    ps.updateXProjection()
    ps.integrate()
    fill = np.asarray(ps.getBunchPopulation(), np.float64)
    total = ps.getIntegral()
    delta = C.c_float()
    _lib.lib().vfps_ps_axis(ps.handle, 0, None, C.byref(delta), None)
    ptr = _lib.lib().vfps_ps_device_data(ps.handle)
    for call in range(2):
        rc, got = noalloc(gpu_ctx, ptr, nb, n, delta.value)
        assert rc == 0, (call, _lib.lib().vfps_last_error(gpu_ctx.handle))
        assert np.allclose(got, fill, rtol=1e-6, atol=0), (call, got, fill)
        s = 0.0
        for v in got:
            s += v
        assert abs(s - total) <= 1e-12 * abs(total), (call, s, total)
    assert gpu_ctx.device_status() == 0


def test_charge_noalloc_rejects_oversize(gpu_ctx):
    ps = V.PhaseSpace(-6.0, 6.0, 1.0, -6.0, 6.0, 1.0, gpu_ctx, n=64)
    ptr = _lib.lib().vfps_ps_device_data(ps.handle)
    # checked before anything is launched: the pointer is never read
    for nb, n in ((4097, 64), (2, 131072 + 1)):
        rc, _ = noalloc(gpu_ctx, ptr, nb, n, 0.1)
        assert rc == _lib.VFPS_ERR_INVALID_ARGUMENT
        msg = _lib.lib().vfps_last_error(gpu_ctx.handle).decode()
        assert "scratch" in msg
