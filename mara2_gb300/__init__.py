"""GB300-native finite-volume time step of Mara2.

The compute path is hand-written CUDA for sm_103a behind a C ABI
(include/mara_gpu.h); this package holds the host-side API over it:

* ``Scheme``   -- the choices a Mara2 driver wires into MethodOfLinesTVD
* ``Solver``   -- one resident grid advanced on the GPU (plain FP64 or mixed)
* ``workloads`` -- seeded synthetic initial data of the benchmark workloads
"""
from .scheme import Scheme  # noqa: F401

__all__ = ["Scheme"]
