"""hydrothermal3d_gb300 -- GB300-native (sm_103a) CUDA implementation of the
HydroThermal3D pseudo-transient hot path behind the C ABI of libht3d.so.

The Python layer mirrors the reference's ParallelStencil kernel interface
(``api``), provides the problem set-up of the benchmark workloads (``hrl``)
and binds the ABI structs (``abi``).  All arithmetic runs in libht3d.so on the
GPU; importing the kernels without the built library raises ImportError.
"""
from . import abi  # noqa: F401
from .api import (Context, Ht3dError, zeros, ones, from_numpy, to_numpy)  # noqa: F401
from . import api  # noqa: F401
from . import hrl  # noqa: F401

__all__ = ["abi", "api", "hrl", "Context", "Ht3dError", "zeros", "ones", "from_numpy", "to_numpy"]
