"""mcgpu_gb300 -- GB300-native Metropolis trial-move energy path of MCGPU.

The CUDA library (``libmcgpu_gb300.so``, built from ``csrc/`` for sm_103a)
does the work; this package is the host side above its C ABI:

* ``step``       the SimulationStep contract (plain single chain, host RNG)
* ``batch``      device-resident batched chains (Philox RNG, on-device accept)
* ``workloads``  seeded synthetic boxes in the SimBox row layout
"""
from . import _abi
from . import files
from ._abi import (PREC_FP64, PREC_MIXED, ROT_AXIS, ROT_EULER, MCGPUError)
from .workloads import BoxData, Topology, bicyclic_box, water_box, water_chains
from .step import Context, GpuBox, GpuSimulationStep, LibcRand, run_plain, run_plain_device_many
from .batch import ChainBatch
from .server import JobServer

__all__ = [
    "PREC_FP64", "PREC_MIXED", "ROT_AXIS", "ROT_EULER", "MCGPUError", "BoxData",
    "bicyclic_box", "water_box", "water_chains", "Context", "GpuBox", "GpuSimulationStep",
    "LibcRand", "run_plain", "run_plain_device_many", "Topology", "ChainBatch", "JobServer",
]
