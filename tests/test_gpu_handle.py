"""The handle API (mc_create ... mc_destroy) against the Python entry points
that keep the reference's interface: same kernels, same streams, so the
results are bit-identical."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def lib():
    from mcgb import _lib
    return _lib, _lib.load()


class Handle:
    def __init__(self, model_id, Ls, temps, seed, **params):
        self._lib, self.lib = lib()
        sig = params.pop("sigmas", None)
        self._sig = None if sig is None else np.ascontiguousarray(sig, np.float32)
        p = self._lib.MCParams(**params)
        if self._sig is not None:
            p.sigmas = self._sig.ctypes.data
        self.Ls = np.ascontiguousarray(Ls, np.int32)
        self.temps = np.ascontiguousarray(temps, np.float64)
        self.h = ctypes.c_void_p()
        self.ok(self.lib.mc_create(model_id, ctypes.byref(p), self.Ls.ctypes.data, len(self.Ls),
                                   self.temps.ctypes.data, seed, None, ctypes.byref(self.h)))

    def ok(self, st):
        assert st == 0, self._lib.last_error()

    def put(self, which, arr):
        arr = np.ascontiguousarray(arr)
        self.ok(self.lib.mc_copy_in(self.h, which, arr.ctypes.data, arr.nbytes))

    def get(self, which, dtype, shape):
        out = np.empty(shape, dtype)
        self.ok(self.lib.mc_copy_out(self.h, which, out.ctypes.data, out.nbytes))
        return out

    def close(self):
        self.ok(self.lib.mc_destroy(self.h))


def test_ising_sweeps_equal_the_runtime():
    from mcgb import _lib
    from mcgb.core.runtime import Runtime
    from mcgb.models.ising.model import IsingModel
    L, temps, seed = 16, [1.8, 2.3, 3.0], 77
    init = np.random.default_rng(1).choice(np.array([-1, 1], np.int8), (3, L, L))
    h = Handle(0, [L] * 3, temps, seed, J=1.0)
    assert (h.get(_lib.MC_STATE, np.int8, (3, L, L)) == 1).all()  # the ordered start
    h.put(_lib.MC_STATE, init)
    h.ok(h.lib.mc_sweep(h.h, 7))
    h.ok(h.lib.mc_update_color(h.h, 2))
    rt = Runtime(IsingModel(J=1.0), L, temps, seed=seed)
    rt.state.copy_to_device(init)
    for _ in range(7):
        rt.sweep()
    rt.model.update_color(rt.state, rt.rng_states, rt.betas, 2, rt.blocks_per_grid, rt.threads_per_block)
    np.testing.assert_array_equal(h.get(_lib.MC_STATE, np.int8, (3, L, L)), rt.snapshot())
    rng = h.get(_lib.MC_RNG, np.uint64, (3 * L * L, 2))
    ref = rt.rng_states.copy_to_host()
    np.testing.assert_array_equal(rng[:, 0], ref["s0"])
    np.testing.assert_array_equal(rng[:, 1], ref["s1"])
    assert h.lib.mc_get_error(h.h) == 0
    h.close()


@pytest.mark.parametrize("gaussian", [False, True])
def test_xy_sweeps_energy_and_measure_equal_the_runtime(gaussian):
    from mcgb import _lib, device
    from mcgb.core.runtime import Runtime
    from mcgb.models.xy.model import XYModel
    L, temps, seed = 16, [0.8, 1.0, 1.2, 1.4], 5
    init = np.random.default_rng(2).uniform(-np.pi, np.pi, (4, L, L)).astype(np.float32)
    sig = np.array([0.6, 0.8, 1.0, 1.2], np.float32)
    kw = dict(J=1.0, delta=1.5)
    if gaussian:
        kw["sigmas"] = sig
    h = Handle(1, [L] * 4, temps, seed, **kw)
    h.put(_lib.MC_STATE, init)
    h.ok(h.lib.mc_sweep(h.h, 5))
    rt = Runtime(XYModel(J=1.0, delta=1.5), L, temps, seed=seed)
    rt.state.copy_to_device(init)
    for _ in range(5):
        for c in range(4):
            if gaussian:
                _lib.call("mcgb_xy_update_color_gauss", rt.state.ptr, rt.rng_states.ptr, rt.betas.ptr,
                          device.to_device(sig).ptr, 4, L, c, ctypes.c_float(1.0), _lib.stream_handle())
            else:
                rt.model.update_color(rt.state, rt.rng_states, rt.betas, c, rt.blocks_per_grid,
                                      rt.threads_per_block)
    np.testing.assert_array_equal(h.get(_lib.MC_STATE, np.float32, (4, L, L)), rt.snapshot())
    h.ok(h.lib.mc_energy(h.h, None))
    energies = h.get(_lib.MC_ENERGIES, np.float64, 4)
    ref_e = device.device_zeros(4, np.float64)
    rt.measure_energy(ref_e)
    np.testing.assert_array_equal(energies, ref_e.copy_to_host())
    tidx = device.to_device(np.array([2, 0, 3, 1], np.int32))
    out = device.device_zeros((5, 4), np.float64)
    h.ok(h.lib.mc_measure(h.h, tidx.ptr, None, out.ptr))
    want = rt.model.measure(rt.state, tidx)
    assert list(want) == ["energy", "mx", "my", "twist_cos_x", "twist_sin_x"]
    for c, name in enumerate(want):
        np.testing.assert_array_equal(out.copy_to_host()[c], want[name], err_msg=name)
    h.close()


def test_ragged_handle_runs_each_size_on_its_own_streams():
    """Replicas of two sizes: each run equals a uniform handle given the same
    streams; measure in temperature order scatters across runs."""
    from mcgb import _lib, device
    Ls, temps = [16, 16, 24, 24, 24], [0.8, 0.9, 1.0, 1.1, 1.2]
    rng = np.random.default_rng(3)
    a = rng.uniform(-np.pi, np.pi, (2, 16, 16)).astype(np.float32)
    b = rng.uniform(-np.pi, np.pi, (3, 24, 24)).astype(np.float32)
    h = Handle(1, Ls, temps, 11, J=1.0, delta=1.5)
    h.put(_lib.MC_STATE, np.concatenate([a.ravel(), b.ravel()]))
    streams = h.get(_lib.MC_RNG, np.uint64, (2 * 256 + 3 * 576, 2))
    h.ok(h.lib.mc_sweep(h.h, 3))
    got = h.get(_lib.MC_STATE, np.float32, 2 * 256 + 3 * 576)
    for (L, init, s0, n, T) in ((16, a, 0, 2, temps[:2]), (24, b, 512, 3, temps[2:])):
        u = Handle(1, [L] * n, T, 99, J=1.0, delta=1.5)
        u.put(_lib.MC_STATE, init)
        u.put(_lib.MC_RNG, streams[s0:s0 + n * L * L])
        u.ok(u.lib.mc_sweep(u.h, 3))
        np.testing.assert_array_equal(got[s0:s0 + n * L * L], u.get(_lib.MC_STATE, np.float32, n * L * L))
        u.close()
    perm = np.array([4, 2, 0, 1, 3], np.int32)
    out = device.device_zeros((5, 5), np.float64)
    h.ok(h.lib.mc_measure(h.h, device.to_device(perm).ptr, None, out.ptr))
    plain = device.device_zeros((5, 5), np.float64)
    h.ok(h.lib.mc_measure(h.h, None, None, plain.ptr))
    np.testing.assert_array_equal(out.copy_to_host()[:, perm], plain.copy_to_host())
    h.close()


def test_exchange_rounds_equal_parallel_tempering():
    from mcgb import _lib
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.models.ising.model import IsingModel
    L, temps, seed = 16, list(np.geomspace(1.8, 3.0, 6)), 21
    init = np.random.default_rng(4).choice(np.array([-1, 1], np.int8), (6, L, L))
    h = Handle(0, [L] * 6, temps, seed, J=1.0)
    h.put(_lib.MC_STATE, init)
    rt = Runtime(IsingModel(J=1.0), L, temps, seed=seed)
    rt.state.copy_to_device(init)
    pt = ParallelTempering(rt, exchange_interval=2)
    for k in range(8):
        h.ok(h.lib.mc_sweep(h.h, 2))
        h.ok(h.lib.mc_exchange(h.h, k % 2, 2 * (k + 1)))
        pt.sweep()
        pt.sweep()
    d = pt.diagnostics()
    np.testing.assert_array_equal(h.get(_lib.MC_W2T, np.int32, 6), d["walker_to_temperature"])
    np.testing.assert_array_equal(h.get(_lib.MC_T2W, np.int32, 6), d["temperature_to_walker"])
    counts = h.get(_lib.MC_SWAP_COUNTS, np.int64, (3, 5))
    np.testing.assert_array_equal(counts[0], d["attempts"])
    np.testing.assert_array_equal(counts[1], d["accepted"])
    np.testing.assert_array_equal(h.get(_lib.MC_STATE, np.int8, (6, L, L)), rt.snapshot())
    h.close()


def test_bad_calls_report_through_the_handle():
    from mcgb import _lib
    h = Handle(0, [16, 16], [1.0, 2.0], 1, J=1.0)
    assert h.lib.mc_update_color(h.h, 7) == _lib.EINVAL
    assert h.lib.mc_get_error(h.h) == _lib.EINVAL and "color" in _lib.last_error()
    assert h.lib.mc_exchange(h.h, 2, 0) == _lib.EINVAL
    buf = np.zeros(3, np.int8)
    assert h.lib.mc_copy_out(h.h, _lib.MC_STATE, buf.ctypes.data, buf.nbytes) == _lib.EINVAL
    h.ok(h.lib.mc_sweep(h.h, 1))
    assert h.lib.mc_get_error(h.h) == 0
    h.close()
