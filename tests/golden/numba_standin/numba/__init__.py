"""A pure-Python stand-in for the part of Numba that the reference's CUDA
kernels use -- fixture-generation infrastructure, never imported by the
product or by any test.

Numba is absent from every machine of this project, so the reference's
kernels (models/*/update.py, models/*/measure.py, models/he3/gaussian_fast.py,
core/parallel_tempering.py) cannot be compiled.  They are plain Python over a
small API: ``cuda.jit``, ``cuda.grid``, ``threadIdx``/``blockIdx``/
``blockDim``, ``cuda.syncthreads``, ``cuda.shared.array``/``cuda.local.array``,
``cuda.to_device``/``device_array``, the scalar types ``float32``/``float64``/
``complex64``, and ``numba.cuda.random``'s xoroshiro128+ streams.  This
package provides that API on the CPU so that the reference's own modules run
UNMODIFIED (``tests/golden/make_reference_kernel_golden.py`` puts this
directory first on ``sys.path``):

* scalar types are NumPy scalars, whose float32 / complex64 arithmetic is
  IEEE single precision like the compiled kernels' (the reference writes its
  float32 constants as ``float32(...)``, so NumPy's promotion of weak Python
  literals never comes into play in the update kernels);
* ``math.*`` inside a jitted function is typed like Numba types it: a
  float32 argument gives a float32 result (CUDA's ``expf``, ``cosf``, ...),
  here the float64 value rounded to float32; float64 arguments give float64.
  ``math.exp`` of a float32 argument whose value CUDA's ``expf`` was
  recorded for (``set_expf_table``) returns that recorded value, so the Ising
  acceptance comparisons see exactly what the GPU computes;
* a kernel launch runs every thread of every block; a kernel that calls
  ``cuda.syncthreads`` (directly or in a device function) runs the threads of
  a block as Python threads meeting at a ``threading.Barrier``, every other
  kernel runs them one after another (the reference's colour kernels touch
  disjoint sites, so the order cannot matter).

Where this differs from the compiled kernels: transcendentals are the
correctly rounded float32 values (CUDA's are within 2 ulp), and NVVM may
contract ``a * b + c`` into an FMA where NumPy rounds twice -- differences
of order 1e-7 relative in continuous states, which the fixtures' consumers
tolerate; integer work, the RNG and the Ising chain are exact.
"""

import numpy as np

float32 = np.float32
float64 = np.float64
complex64 = np.complex64
complex128 = np.complex128
int8 = np.int8
int16 = np.int16
int32 = np.int32
int64 = np.int64
uint32 = np.uint32
uint64 = np.uint64
boolean = np.bool_

from . import cuda  # noqa: E402,F401

__version__ = "0.0-standin"
