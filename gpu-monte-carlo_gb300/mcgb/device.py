"""Device arrays: torch CUDA allocations with the array semantics the
reference's host code relies on.

The reference holds device state in Numba device arrays and its tests use
``copy_to_device``, ``copy_to_host``, ``shape``, ``dtype``, ``size`` and
slicing (core/runtime.py:47-57, core/parallel_tempering.py:151-225,
tests/test_simulation.py:113).  :class:`DeviceArray` offers that surface over
a raw byte allocation made by torch's caching allocator; torch is only the
memory and stream carrier, all compute is in ``libmcgb.so``.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

# numba.cuda.random.xoroshiro128p_dtype: two uint64 words per stream.
XOROSHIRO128P_DTYPE = np.dtype([("s0", np.uint64), ("s1", np.uint64)], align=True)

_TORCH_DTYPES = {
    np.dtype(np.int8): torch.int8,
    np.dtype(np.uint8): torch.uint8,
    np.dtype(np.int32): torch.int32,
    np.dtype(np.int64): torch.int64,
    np.dtype(np.float32): torch.float32,
    np.dtype(np.float64): torch.float64,
    np.dtype(np.complex64): torch.complex64,
}


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("mcgb requires a CUDA GPU; none is available")
    return torch.device("cuda", torch.cuda.current_device())


class DeviceArray:
    """A C-contiguous device array of a NumPy dtype, backed by torch bytes."""

    def __init__(self, shape, dtype, _storage=None):
        self.dtype = np.dtype(dtype)
        self.shape = tuple(int(s) for s in (shape if isinstance(shape, (tuple, list)) else (shape,)))
        nbytes = int(np.prod(self.shape, dtype=np.int64)) * self.dtype.itemsize
        if _storage is None:
            _storage = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=_device())
        self._t = _storage
        self._nbytes = nbytes

    # ------------------------------------------------------------ metadata
    @property
    def size(self):
        return int(np.prod(self.shape, dtype=np.int64))

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def nbytes(self):
        return self._nbytes

    @property
    def ptr(self) -> int:
        return self._t.data_ptr()

    @property
    def cptr(self):
        return ctypes.c_void_p(self._t.data_ptr())

    def __len__(self):
        return self.shape[0]

    def __repr__(self):
        return f"DeviceArray(shape={self.shape}, dtype={self.dtype})"

    @property
    def __cuda_array_interface__(self):
        return {
            "shape": self.shape,
            "typestr": self.dtype.str if self.dtype.fields is None else "|V%d" % self.dtype.itemsize,
            "data": (self.ptr, False),
            "version": 3,
            "strides": None,
        }

    # ------------------------------------------------------------ views
    def raw(self):
        """The array's bytes as a flat uint8 torch tensor (no copy)."""
        return self._t[: self._nbytes]

    def torch(self, dtype=None):
        """Typed torch view of the same memory (no copy); array-shaped when the
        element size matches, else flat."""
        if dtype is None:
            dtype = _TORCH_DTYPES[self.dtype]
        view = self.raw().view(dtype)
        if self.dtype.fields is None and view.element_size() == self.dtype.itemsize:
            return view.view(self.shape)
        return view

    def __getitem__(self, key):
        """Contiguous slices along axis 0 (``chunk[:used]``, ``arr[3]``)."""
        n = self.shape[0]
        row = self._nbytes // n if n else 0
        if isinstance(key, slice):
            start, stop, step = key.indices(n)
            if step != 1:
                raise IndexError("DeviceArray supports unit-step slices only")
            stop = max(stop, start)
            storage = self._t[start * row: stop * row] if stop > start else self._t[:0]
            return DeviceArray((stop - start,) + self.shape[1:], self.dtype, _storage=storage)
        if isinstance(key, (int, np.integer)):
            k = int(key) + (n if key < 0 else 0)
            if not 0 <= k < n:
                raise IndexError("index out of range")
            return DeviceArray(self.shape[1:], self.dtype, _storage=self._t[k * row:(k + 1) * row])
        raise IndexError("unsupported DeviceArray index")

    # ------------------------------------------------------------ copies
    def copy_to_device(self, ary, stream=None):
        """Copy a host array of the same size into this array (synchronously)."""
        host = np.ascontiguousarray(np.asarray(ary, dtype=self.dtype))
        if host.size != self.size:
            raise ValueError(f"copy_to_device: size {host.size} does not match {self.size}")
        src = torch.from_numpy(host.reshape(-1).view(np.uint8).copy())
        self._t[: self._nbytes].copy_(src)
        return self

    def copy_to_host(self, ary=None, stream=None):
        """Return (or fill ``ary`` with) a host copy; waits for pending work."""
        data = self._t[: self._nbytes].cpu().numpy().view(self.dtype).reshape(self.shape)
        if ary is not None:
            ary[...] = data
            return ary
        return data

    def copy_to_host_async(self):
        """Non-blocking copy into pinned memory; returns (array, event)."""
        pinned = torch.empty(self._nbytes, dtype=torch.uint8, pin_memory=True)
        pinned.copy_(self._t[: self._nbytes], non_blocking=True)
        event = torch.cuda.Event()
        event.record()
        return pinned.numpy().view(self.dtype).reshape(self.shape), event

    def fill_zero(self):
        self._t[: self._nbytes].zero_()
        return self


def to_device(ary, dtype=None) -> DeviceArray:
    host = np.ascontiguousarray(ary if dtype is None else np.asarray(ary, dtype=dtype))
    out = DeviceArray(host.shape, host.dtype)
    return out.copy_to_device(host)


def device_array(shape, dtype=np.float64) -> DeviceArray:
    return DeviceArray(shape, dtype)


def device_zeros(shape, dtype=np.float64) -> DeviceArray:
    return DeviceArray(shape, dtype).fill_zero()


def ptr(a):
    """ctypes pointer of a DeviceArray / torch tensor / None."""
    if a is None:
        return None
    if isinstance(a, DeviceArray):
        return a.cptr
    if isinstance(a, torch.Tensor):
        if not a.is_cuda or not a.is_contiguous():
            raise ValueError("expected a contiguous CUDA tensor")
        return ctypes.c_void_p(a.data_ptr())
    iface = getattr(a, "__cuda_array_interface__", None)
    if iface is not None:
        return ctypes.c_void_p(iface["data"][0])
    raise TypeError(f"not a device array: {type(a).__name__}")


def synchronize():
    torch.cuda.current_stream().synchronize()
