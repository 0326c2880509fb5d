"""``numba.cuda`` on the CPU: kernel launches, thread indices, barriers,
shared/local arrays and device arrays (see the package docstring)."""

import math as _math
import threading
import types

import numpy as np

# ------------------------------------------------------------ device arrays


class DeviceNDArray(np.ndarray):
    """Host memory standing in for a device array (copy_to_host/device)."""

    def copy_to_host(self, ary=None, stream=0):
        host = np.array(self.view(np.ndarray), copy=True)
        if ary is not None:
            ary[...] = host
            return ary
        return host

    def copy_to_device(self, ary, stream=0):
        self.view(np.ndarray)[...] = np.asarray(ary)

    def is_c_contiguous(self):
        return self.flags.c_contiguous


def to_device(obj, stream=0, copy=True, to=None):
    host = np.array(obj, copy=True)
    if to is not None:
        to.copy_to_device(host)
        return to
    return host.view(DeviceNDArray)


def device_array(shape, dtype=np.float64, strides=None, order="C", stream=0):
    return np.zeros(shape, dtype=dtype, order=order).view(DeviceNDArray)


def device_array_like(ary, stream=0):
    return device_array(ary.shape, ary.dtype)


def synchronize():
    return None


def is_available():
    return True


# ------------------------------------------------------------ typed math

_F32 = np.float32
_F64 = np.float64
_expf_table = {}
_expf_misses = set()


def set_expf_table(table):
    """Record CUDA's expf values: {float32 argument bits: float32 result bits}."""
    _expf_table.clear()
    _expf_table.update({int(k): int(v) for k, v in table.items()})


def expf_misses():
    """float32 arguments of math.exp evaluated without a recorded CUDA value."""
    return set(_expf_misses)


def clear_expf_misses():
    _expf_misses.clear()


def _all_f32(args):
    return all(isinstance(a, (np.float32, np.complex64)) for a in args)


def _typed(name):
    fn = getattr(np, name)

    def wrapped(*args):
        with np.errstate(all="ignore"):
            if _all_f32(args):
                return _F32(fn(*[_F64(a) for a in args]))
            return _F64(fn(*[_F64(a) for a in args]))
    wrapped.__name__ = name
    return wrapped


def _exp(x):
    with np.errstate(all="ignore"):
        if isinstance(x, np.float32):
            bits = int(np.asarray(x).view(np.uint32))
            if bits in _expf_table:
                return np.array(_expf_table[bits], np.uint32).view(np.float32)[()]
            _expf_misses.add(bits)
            return _F32(np.exp(_F64(x)))
        return _F64(np.exp(_F64(x)))


def _isfinite(x):
    return bool(np.isfinite(x))


def _isnan(x):
    return bool(np.isnan(x))


def _isinf(x):
    return bool(np.isinf(x))


class _TypedMath(types.ModuleType):
    """``math`` as Numba types it inside kernels (float32 in, float32 out)."""

    def __getattr__(self, name):
        return getattr(_math, name)


typed_math = _TypedMath("math")
for _name, _np in (("cos", "cos"), ("sin", "sin"), ("tan", "tan"), ("log", "log"), ("sqrt", "sqrt"),
                   ("atan2", "arctan2"), ("atan", "arctan"), ("acos", "arccos"), ("asin", "arcsin"),
                   ("fabs", "fabs"), ("tanh", "tanh"), ("log1p", "log1p"), ("expm1", "expm1"),
                   ("cosh", "cosh"), ("sinh", "sinh"), ("hypot", "hypot")):
    setattr(typed_math, _name, _typed(_np))
typed_math.exp = _exp
typed_math.isfinite = _isfinite
typed_math.isnan = _isnan
typed_math.isinf = _isinf

# ------------------------------------------------------------ thread context

_tls = threading.local()


class _Dim3Proxy:
    def __init__(self, field):
        self._field = field

    @property
    def x(self):
        return getattr(_tls, self._field)[0]

    @property
    def y(self):
        return getattr(_tls, self._field)[1]

    @property
    def z(self):
        return getattr(_tls, self._field)[2]


threadIdx = _Dim3Proxy("tid")
blockIdx = _Dim3Proxy("bid")
blockDim = _Dim3Proxy("bdim")
gridDim = _Dim3Proxy("gdim")


def grid(ndim):
    t, b, d = _tls.tid, _tls.bid, _tls.bdim
    g = tuple(t[k] + b[k] * d[k] for k in range(3))
    return g[0] if ndim == 1 else g[:ndim]


def gridsize(ndim):
    d, n = _tls.bdim, _tls.gdim
    g = tuple(d[k] * n[k] for k in range(3))
    return g[0] if ndim == 1 else g[:ndim]


def syncthreads():
    barrier = getattr(_tls, "barrier", None)
    if barrier is None:
        raise RuntimeError("syncthreads outside a barrier-synchronised launch")
    barrier.wait()


class _Block:
    def __init__(self):
        self.lock = threading.Lock()
        self.shared = []


class _Shared:
    @staticmethod
    def array(shape, dtype):
        block, k = _tls.block, _tls.shared_calls
        _tls.shared_calls = k + 1
        with block.lock:
            if k == len(block.shared):
                block.shared.append(np.zeros(shape, dtype=dtype))
            return block.shared[k]


class _Local:
    @staticmethod
    def array(shape, dtype):
        return np.zeros(shape, dtype=dtype)


shared = _Shared()
local = _Local()

# ------------------------------------------------------------ jit and launch


def _install_typed_math(fn):
    g = fn.__globals__
    if g.get("math") is _math:
        g["math"] = typed_math


def _uses_barrier(fn, seen=None):
    seen = set() if seen is None else seen
    if fn in seen:
        return False
    seen.add(fn)
    codes = [fn.__code__]
    names = set()
    while codes:
        c = codes.pop()
        names.update(c.co_names)
        codes.extend(k for k in c.co_consts if isinstance(k, types.CodeType))
    if "syncthreads" in names:
        return True
    for name in names:
        obj = fn.__globals__.get(name)
        if getattr(obj, "_standin_device", False) and _uses_barrier(obj, seen):
            return True
    return False


def _dim3(v):
    if isinstance(v, (tuple, list)):
        v = tuple(int(x) for x in v) + (1,) * (3 - len(v))
        return v[:3]
    return (int(v), 1, 1)


def _host_view(a):
    return a.view(np.ndarray) if isinstance(a, DeviceNDArray) else a


class _Kernel:
    def __init__(self, fn):
        _install_typed_math(fn)
        self.py_func = fn
        self.__name__ = fn.__name__
        self._barrier = None

    def __getitem__(self, config):
        blocks, threads = config[0], config[1]
        return lambda *args: self._launch(_dim3(blocks), _dim3(threads), args)

    def _run_thread(self, tid, bid, bdim, gdim, block, barrier, args, errors):
        _tls.tid, _tls.bid, _tls.bdim, _tls.gdim = tid, bid, bdim, gdim
        _tls.block, _tls.shared_calls, _tls.barrier = block, 0, barrier
        try:
            self.py_func(*args)
        except BaseException as e:  # surface it in the launching thread
            errors.append(e)
            if barrier is not None:
                barrier.abort()
        finally:
            _tls.barrier = None

    def _launch(self, gdim, bdim, args):
        if self._barrier is None:
            self._barrier = _uses_barrier(self.py_func)
        args = tuple(_host_view(a) for a in args)
        n = bdim[0] * bdim[1] * bdim[2]
        tids = [(x, y, z) for z in range(bdim[2]) for y in range(bdim[1]) for x in range(bdim[0])]
        saved = {k: getattr(_tls, k, None) for k in ("tid", "bid", "bdim", "gdim", "block", "shared_calls",
                                                        "barrier")}
        try:
            for bz in range(gdim[2]):
                for by in range(gdim[1]):
                    for bx in range(gdim[0]):
                        bid, block, errors = (bx, by, bz), _Block(), []
                        if not self._barrier:
                            for tid in tids:
                                self._run_thread(tid, bid, bdim, gdim, block, None, args, errors)
                                if errors:
                                    raise errors[0]
                            continue
                        barrier = threading.Barrier(n)
                        workers = [threading.Thread(target=self._run_thread,
                                                    args=(tid, bid, bdim, gdim, block, barrier, args, errors))
                                   for tid in tids]
                        for w in workers:
                            w.start()
                        for w in workers:
                            w.join()
                        real = [e for e in errors if not isinstance(e, threading.BrokenBarrierError)]
                        if real or errors:
                            raise (real or errors)[0]
        finally:
            for k, v in saved.items():
                setattr(_tls, k, v)


def jit(fn=None, device=False, **options):
    """``@cuda.jit`` (a kernel) and ``@cuda.jit(device=True)`` (a device function)."""
    def wrap(f):
        if device:
            _install_typed_math(f)
            f._standin_device = True
            return f
        return _Kernel(f)
    if callable(fn):
        return wrap(fn)
    return wrap


from . import random  # noqa: E402,F401
