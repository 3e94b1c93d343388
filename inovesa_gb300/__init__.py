"""GB300-native phase-space hot path of the Inovesa Vlasov-Fokker-Planck
solver: CUDA kernels for sm_103a behind the C ABI of include/vfps.h
(libvfps.so), with a Python mirror of the reference's classes in
:mod:`inovesa_gb300.vfps` and physics-parameter derivation in
:mod:`inovesa_gb300.params`.
"""
from . import build  # noqa: F401

__all__ = ["build", "vfps", "params"]
