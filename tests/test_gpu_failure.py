"""Failure detection without a GPU fault.

* A bounded wait that runs out: a kernel walks 16 tiles waiting on
  barriers that nothing completes (vfps_selftest_wait_timeout, the wait
  pattern of the persistent solver kernels); the first wait gives up after
  its limit and the CTA stops walking, so the call ends after about two
  limits rather than two per tile; the device status reads
  VFPS_ERR_TIMEOUT, and the context keeps working (a batch steps cleanly
  afterwards).
* The charge watchdog of the batched step: a bunch whose density carries
  no charge sets VFPS_ERR_NUMERIC (the reference throws on an
  unnormalisable filling, src/PS/PhaseSpace.cpp:47-51); after a valid
  upload the batch steps cleanly again."""
import time

import numpy as np
import pytest

from inovesa_gb300 import _lib
from inovesa_gb300 import params as P
from inovesa_gb300 import vfps as V

pytestmark = pytest.mark.gpu


def small_batch(ctx):
    p = P.derive(GridSize=64, StepsPerTs=200, padding=2.0, VacuumGap=0.0318,
                 S_csr=0.3)
    z = V.makeImpedance(ctx, **P.wake_impedance_args(p))
    d = P.fill_desc(V.BunchDesc(), p, 0, Ib=p["Ib"], impedance=0)
    return V.BunchBatch(ctx, [d, d], [z])


def test_bounded_wait_reports_timeout(gpu_ctx):
    assert gpu_ctx.device_status() == 0
    t0 = time.perf_counter()
    _lib.check(_lib.lib().vfps_selftest_wait_timeout(gpu_ctx.handle,
                                                     2_000_000),
               gpu_ctx.handle)
    assert time.perf_counter() - t0 < 5.0
    assert gpu_ctx.device_status() == _lib.VFPS_ERR_TIMEOUT
    # 100 ms limits: 16 tiles of two waits each would take 3.2 s; the
    # early exit ends the walk after the first tile's two waits
    t0 = time.perf_counter()
    _lib.check(_lib.lib().vfps_selftest_wait_timeout(gpu_ctx.handle,
                                                     100_000_000),
               gpu_ctx.handle)
    el = time.perf_counter() - t0
    assert 0.19 < el < 1.0, el
    assert gpu_ctx.device_status() == _lib.VFPS_ERR_TIMEOUT
    assert gpu_ctx.device_status() == 0          # reading cleared it
    b = small_batch(gpu_ctx)
    b.step(10)
    assert gpu_ctx.device_status() == 0
    with pytest.raises(V.VfpsError):
        _lib.check(_lib.lib().vfps_selftest_wait_timeout(gpu_ctx.handle, 0),
                   gpu_ctx.handle)


def test_charge_watchdog(gpu_ctx):
    b = small_batch(gpu_ctx)
    good = b.download()
    b.upload(np.zeros_like(good))
    b.step(1)
    assert gpu_ctx.device_status() == _lib.VFPS_ERR_NUMERIC
    b.upload(good)
    b.step(5)
    assert gpu_ctx.device_status() == 0
    assert np.all(np.isfinite(b.download()))
