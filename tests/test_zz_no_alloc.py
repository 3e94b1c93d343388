"""vfps_charge_noalloc (charge integrals from raw device pointers, no
allocation) against the PhaseSpace path that owns its buffers
(vfps_ps_update_x_projection + vfps_ps_integrate).

Collected last (file name) so that it also runs after every other GPU
test in the same process; it passes alone in a fresh process too.
Tolerance: both paths add in the same order, so the FP64 integrals agree
to 1e-12 relative; the PhaseSpace path hands per-bunch values out as
float, compared at 1e-6 relative.  The calls at the scratch's limits are
compared with an FP64 NumPy Simpson sum of the same data at 1e-6 relative
(the device sums groups of 8 cells in FP32).  The property that makes the
entry point worth having, that it allocates nothing, is checked through
the device's free memory: unchanged across calls after the first.
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


def simpson_charges(data, delta):
    """FP64 Simpson integrals of meshes [nb][n][n] with the PhaseSpace
    path's float weights (delta/3 at both ends, times 4 at odd and 2 at
    even interior indices)."""
    n = data.shape[-1]
    h03 = np.float32(delta) / np.float32(3)
    ws = np.where(np.arange(n) % 2 == 1, h03 * np.float32(4),
                  h03 * np.float32(2)).astype(np.float32)
    ws[0] = ws[-1] = h03
    w = ws.astype(np.float64)
    proj = data.astype(np.float64) @ w
    return proj @ w


@pytest.mark.parametrize("nb,n", [(1024, 256), (4096, 64)])
def test_charge_noalloc_at_the_limits(gpu_ctx, nb, n):
    """The largest accepted calls: every row of the scratch, and (4096
    meshes) every per-mesh result slot; the device's free memory does not
    change across the calls."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(nb + n)
    data = rng.random((nb, n, n), dtype=np.float32)
    dev = torch.from_numpy(data).to("cuda:0")
    torch.cuda.synchronize()
    delta = 12.0 / (n - 1)
    want = simpson_charges(data, delta)
    rc, got = noalloc(gpu_ctx, dev.data_ptr(), nb, n, delta)
    assert rc == 0, _lib.lib().vfps_last_error(gpu_ctx.handle)
    free0, _ = torch.cuda.mem_get_info(0)
    for call in range(2):
        rc, got = noalloc(gpu_ctx, dev.data_ptr(), nb, n, delta)
        assert rc == 0, (call, _lib.lib().vfps_last_error(gpu_ctx.handle))
        assert np.allclose(got, want, rtol=1e-6, atol=0), call
        free1, _ = torch.cuda.mem_get_info(0)
        assert free1 == free0, (call, free0, free1)
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
