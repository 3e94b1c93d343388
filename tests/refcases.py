"""Set-ups shared by the oracle and GPU parity tests.

They rebuild, from the golden fixture, the objects the reference's tests
construct (test/TestElectricField.cpp:22-93 for the ElectricField fixture).
"""
import math

import numpy as np

C_LIGHT = 2.99792458e8


def ef_fixture(fx, pattern):
    """Buckets, bunch fillings, spacing and wake scaling of the
    ElectricFieldFixture for one filling pattern."""
    n = fx["n"]
    spacing_bins = int(math.ceil(n * fx["bunchspacing"]))
    spaced_bins = spacing_bins * len(pattern)
    buckets, bunches = [], []
    for i, f in enumerate(pattern):
        if f > 0:
            buckets.append(len(pattern) - 1 - i)
            bunches.append(f)
    axes = fx["axes"]
    dp = np.float32((axes[4] - axes[3]) / np.float32(n - 1))
    dp = np.float32(np.float32(axes[4]) - np.float32(axes[3])) / np.float32(
        n - 1)
    # inc/PS/ElectricField.hpp:99-100, evaluated in double then passed on
    # as float
    wakescaling = (fx["Ib"] * fx["dt"] * C_LIGHT / axes[2]
                   / (float(dp) * fx["sigma_delta"] * fx["E0"]))
    return dict(n=n, spacing=spacing_bins, nmax=spaced_bins, buckets=buckets,
                bunches=bunches, axes=axes, wakescaling=wakescaling)


def gauss_projection(axis, zoom=1.0):
    return (1.0 / math.sqrt(2 * math.pi)) * np.exp(-0.5 * axis * axis
                                                   / (zoom * zoom))
