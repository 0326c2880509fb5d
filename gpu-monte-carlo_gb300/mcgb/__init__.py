"""mcgb: GB300-native lattice Monte Carlo hot path.

Python host code mirroring the reference's plugin interface (``core.model``)
and entry points (``core.runtime.Runtime``, ``core.parallel_tempering``,
``core.simulation``), calling hand-written sm_103a CUDA kernels in
``libmcgb.so`` through a C ABI (ctypes).  PyTorch only carries device memory
and streams.
"""

__version__ = "0.1.0"
