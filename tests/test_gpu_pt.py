"""Parallel tempering, the energy cache and the Simulation loop on the GPU:
ports of tests/test_parallel_tempering.py, tests/test_pt_walkers.py,
tests/test_energy_cache.py and tests/test_simulation.py:137-177."""

from unittest.mock import patch

import numpy as np
import pytest

import npref

pytestmark = pytest.mark.gpu


def constant_xy(angles, exchange_interval=1):
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.models.xy.model import XYModel
    rt = Runtime(XYModel(J=1.37), L=4, temperatures=np.linspace(0.6, 1.4, len(angles)), seed=31)
    state = np.broadcast_to(np.asarray(angles, np.float32)[:, None, None], (len(angles), 4, 4)).copy()
    rt.state.copy_to_device(state)
    return rt, ParallelTempering(rt, exchange_interval=exchange_interval, seed=97), state


def assert_mappings(pt, t2w):
    expected = np.asarray(t2w, np.int32)
    actual = pt.temperature_to_walker.copy_to_host()
    reverse = pt.walker_to_temperature.copy_to_host()
    np.testing.assert_array_equal(actual, expected)
    np.testing.assert_array_equal(reverse[actual], np.arange(pt.R))
    np.testing.assert_array_equal(actual[reverse], np.arange(pt.R))
    ladder = (1.0 / pt.temperatures).astype(np.float32)
    np.testing.assert_array_equal(pt.runtime.betas.copy_to_host(), ladder[reverse])


def test_accepted_exchanges_preserve_walkers_and_order_every_channel():
    rt, pt, state = constant_xy([0.0, 0.5, 1.0, -0.5])
    site_rng = rt.rng_states.copy_to_host()
    ref = npref.xy(state, rt.model.J)
    pt.attempt_exchanges()
    order = np.array([1, 0, 3, 2])
    assert_mappings(pt, order)
    np.testing.assert_array_equal(rt.snapshot(), state)
    np.testing.assert_array_equal(rt.rng_states.copy_to_host(), site_rng)
    np.testing.assert_array_equal(pt.snapshot(), state[order])
    m = pt.measure()
    for name, values in ref.items():
        np.testing.assert_allclose(m[name], values[order], rtol=1e-12, atol=1e-10)
    pt.attempt_exchanges()
    assert_mappings(pt, [1, 3, 0, 2])
    d = pt.diagnostics()
    np.testing.assert_array_equal(d["attempts"], [1, 1, 1])
    np.testing.assert_array_equal(d["accepted"], [1, 1, 1])
    np.testing.assert_array_equal(d["acceptance_rates"], [1.0, 1.0, 1.0])


@pytest.mark.parametrize("R", [5, 259])
def test_alternating_disjoint_pairs_and_more_pairs_than_threads(R):
    _, pt, _ = constant_xy(np.linspace(-1.0, 1.0, R))
    order = np.arange(R)
    attempts = np.zeros(R - 1, np.int64)
    for rnd in range(4):
        for t in range(rnd % 2, R - 1, 2):
            order[t:t + 2] = order[t:t + 2][::-1]
            attempts[t] += 1
        pt.attempt_exchanges()
        assert_mappings(pt, order)
        d = pt.diagnostics()
        np.testing.assert_array_equal(d["attempts"], attempts)
        np.testing.assert_array_equal(d["accepted"], attempts)
        assert d["exchange_rounds"] == rnd + 1


def test_nonfinite_energy_prevents_swap_and_diagnostics_raise():
    rt, pt, state = constant_xy([0.0, 1.0])
    state[0, 0, 0] = np.nan
    rt.state.copy_to_device(state)
    pt.attempt_exchanges()
    assert np.isnan(pt.energies.copy_to_host()[0])
    assert_mappings(pt, [0, 1])
    with pytest.raises(FloatingPointError):
        pt.diagnostics()


def test_acceptance_sign_and_current_total_ising_energies():
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.models.ising.model import IsingModel
    rt = Runtime(IsingModel(J=1.37), L=4, temperatures=[1e-6, 1e6], seed=32)
    pt = ParallelTempering(rt, exchange_interval=1, seed=98)
    ordered = np.ones((4, 4), np.int8)
    cb = (1 - 2 * (np.indices((4, 4)).sum(axis=0) % 2)).astype(np.int8)
    mag = 2 * float(rt.model.J) * 16
    rt.state.copy_to_device(np.stack([ordered, cb]))
    pt.attempt_exchanges()
    np.testing.assert_array_equal(pt.energies.copy_to_host(), [-mag, mag])
    assert_mappings(pt, [0, 1])
    np.testing.assert_array_equal(pt.diagnostics()["accepted"], [0])
    state = np.stack([cb, ordered])
    rt.state.copy_to_device(state)
    pt.attempt_exchanges()
    np.testing.assert_array_equal(pt.energies.copy_to_host(), [mag, -mag])
    assert_mappings(pt, [1, 0])
    np.testing.assert_array_equal(pt.diagnostics()["attempts"], [2])
    np.testing.assert_array_equal(pt.diagnostics()["accepted"], [1])
    m = pt.measure()
    np.testing.assert_array_equal(m["energy"], [-mag, mag])
    np.testing.assert_array_equal(m["magnetization"], [16, 0])
    np.testing.assert_array_equal(rt.snapshot(), state)


def test_xy_exchange_energies_fresh_and_match_cpu_bonds():
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.models.xy.model import XYModel
    rt = Runtime(XYModel(J=1.37), L=6, temperatures=[0.7, 1.0, 1.3], seed=33)
    pt = ParallelTempering(rt, seed=99)
    rng = np.random.default_rng(34)
    for _ in range(2):
        state = rng.uniform(-np.pi, np.pi, (3, 6, 6)).astype(np.float32)
        rt.state.copy_to_device(state)
        ref = npref.xy(state, rt.model.J)
        pt.attempt_exchanges()
        np.testing.assert_allclose(pt.energies.copy_to_host(), ref["energy"], rtol=1e-12, atol=1e-10)
        order = pt.temperature_to_walker.copy_to_host()
        assert_mappings(pt, order)
        m = pt.measure()
        for name, values in ref.items():
            np.testing.assert_allclose(m[name], values[order], rtol=1e-12, atol=1e-10)


def test_exchange_interval_and_round_trips():
    rt, pt, _ = constant_xy([0.0, 1.0], exchange_interval=2)
    assert pt.diagnostics()["mean_round_trip_sweeps"] is None
    with patch.object(rt, "sweep") as sweep:
        for k in range(1, 7):
            pt.sweep()
            assert pt.sweeps == k and pt.diagnostics()["exchange_rounds"] == k // 2
        assert sweep.call_count == 6
    d = pt.diagnostics()
    np.testing.assert_array_equal(d["attempts"], [3])
    np.testing.assert_array_equal(d["walker_round_trips"], [1, 1])
    np.testing.assert_array_equal(d["walker_round_trip_total_sweeps"], [4, 4])
    assert d["mean_round_trip_sweeps"] == 4.0
    rt, pt, _ = constant_xy([0.0, 0.5, 1.0])
    with patch.object(rt, "sweep"):
        for _ in range(6):
            pt.sweep()
        np.testing.assert_array_equal(pt.diagnostics()["walker_round_trips"], [1, 0, 1])
        pt.sweep()
    d = pt.diagnostics()
    np.testing.assert_array_equal(d["walker_round_trips"], [1, 1, 1])
    np.testing.assert_array_equal(d["walker_round_trip_total_sweeps"], [5, 6, 6])


def test_simulation_preserves_temperature_order_and_diagnostics():
    from mcgb.core.simulation import Simulation
    rt, pt, state = constant_xy([0.0, 1.0], exchange_interval=3)
    sim = Simulation(pt, thermalization_sweeps=4, measurement_sweeps=7, sample_interval=2)
    with patch.object(rt, "sweep") as sweep:
        run = sim.run()
    assert sweep.call_count == 11
    np.testing.assert_array_equal(run["metadata"]["sample_sweeps"], [6, 8, 10])
    mx = npref.xy(state, rt.model.J)["mx"]
    np.testing.assert_allclose(run["samples"]["mx"], [mx, mx, mx[::-1]], atol=1e-12)
    d = run["metadata"]["parallel_tempering"]
    assert d["exchange_interval"] == 3 and d["exchange_seed"] == 97
    assert d["sweeps"] == 11 and d["exchange_rounds"] == 3
    np.testing.assert_array_equal(d["attempts"], [3])
    np.testing.assert_array_equal(d["walker_round_trips"], [1, 1])
    assert d["mean_round_trip_sweeps"] == 6.0


def test_invalid_ladders_and_intervals():
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.models.ising.model import IsingModel
    for temps in ([1.0], [1.0, 1.0], [2.0, 1.0], [1.0, 2.0, 1.5], [1.0, 1.0 + 1e-10]):
        with pytest.raises(ValueError):
            ParallelTempering(Runtime(IsingModel(), L=4, temperatures=temps))
    rt = Runtime(IsingModel(), L=4, temperatures=[1.0, 2.0])
    for interval in (0, -1, 1.5, True):
        with pytest.raises(ValueError):
            ParallelTempering(rt, exchange_interval=interval)


# ------------------------------------------------------------ walker history

def make_pt(R=4, **kw):
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.models.xy.model import XYModel
    rt = Runtime(XYModel(), L=4, temperatures=np.linspace(.8, 1.2, R), threads=2, seed=162)
    return rt, ParallelTempering(rt, exchange_interval=1, seed=163, **kw)


def test_history_matches_live_mappings_and_chunk_growth():
    rt, pt = make_pt(tracked_walkers=range(4), history_stride=1)
    pt._history_chunk_rows = 4
    expected = [np.arange(4)]
    with patch.object(rt, "sweep"):
        for _ in range(10):
            pt.sweep()
            expected.append(pt.walker_to_temperature.copy_to_host())
    h = pt.diagnostics()["walker_history"]
    assert len(pt._history_chunks) == 3
    np.testing.assert_array_equal(h["temperature_indices"], expected)
    np.testing.assert_array_equal(h["sweeps"], np.arange(11))
    np.testing.assert_array_equal(h["exchange_rounds"], np.arange(11))


def test_history_stride_final_snapshot_and_manual_exchanges():
    rt, pt = make_pt(tracked_walkers=[3, 0], history_stride=3)
    with patch.object(rt, "sweep"):
        for _ in range(7):
            pt.sweep()
    h = pt.diagnostics()["walker_history"]
    np.testing.assert_array_equal(h["sweeps"], [0, 3, 6, 7])
    np.testing.assert_array_equal(h["temperature_indices"][-1], pt.walker_to_temperature.copy_to_host()[[3, 0]])
    assert len(pt._history_sweeps) == 3
    _, pt2 = make_pt(R=2, tracked_walkers=[0, 1], history_stride=1)
    for _ in range(4):
        pt2.attempt_exchanges()
    d = pt2.diagnostics()
    np.testing.assert_array_equal(d["walker_history"]["sweeps"], 0)
    np.testing.assert_array_equal(d["walker_history"]["temperature_indices"],
                                  [[0, 1], [1, 0], [0, 1], [1, 0], [0, 1]])
    np.testing.assert_array_equal(d["walker_round_trips"], [2, 2])
    _, pt3 = make_pt()
    assert pt3._history_chunks == [] and "walker_history" not in pt3.diagnostics()


# ------------------------------------------------------------ energy cache

def he3_runtime(L=6, R=3):
    from mcgb.core.runtime import Runtime
    from mcgb.models.he3.model import He3Model
    rt = Runtime(He3Model(pressure=20), L=L, temperatures=np.linspace(0.2, 0.5, R), threads=2, seed=211)
    rng = np.random.default_rng(212)
    st = 0.25 * (rng.normal(size=(R, L, L, 3, 2)) + 1j * rng.normal(size=(R, L, L, 3, 2)))
    rt.state.copy_to_device(st.astype(np.complex64))
    rt.invalidate_energy_cache()
    return rt


def cache_energy(rt):
    from mcgb.device import device_array
    e = device_array(rt.R, np.float64)
    rt.measure_energy(e)
    return e


def assert_meas_equal(a, b):
    assert a.keys() == b.keys()
    for k in a:
        np.testing.assert_allclose(a[k], b[k], rtol=2e-6, atol=1e-5)


def test_cached_measurements_match_and_energy_is_readonly():
    rt = he3_runtime()
    expected = rt.model.measure(rt.state)
    e = cache_energy(rt)
    orig = e.copy_to_host()
    with patch.object(rt.model, "measure_with_energy", wraps=rt.model.measure_with_energy) as cached:
        actual = rt.measure()
    cached.assert_called_once()
    assert_meas_equal(actual, expected)
    np.testing.assert_array_equal(actual["energy"], orig)
    np.testing.assert_array_equal(e.copy_to_host(), orig)


def test_sweep_and_explicit_invalidation_and_failures():
    rt = he3_runtime(L=4, R=2)
    old = cache_energy(rt).copy_to_host()
    rt.betas.copy_to_device(np.zeros(rt.R, np.float32))
    rt.sweep()
    with patch.object(rt.model, "measure_with_energy", wraps=rt.model.measure_with_energy) as cached:
        actual = rt.measure()
    cached.assert_not_called()
    assert_meas_equal(actual, rt.model.measure(rt.state))
    assert not np.allclose(actual["energy"], old)

    rt = he3_runtime(L=4, R=2)
    cache_energy(rt)
    changed = (1.2 * rt.snapshot()).astype(np.complex64)

    def fail_after_mutation(*a, **k):
        rt.state.copy_to_device(changed)
        raise RuntimeError("interrupted update")

    with patch.object(rt.model, "update_color", side_effect=fail_after_mutation):
        with pytest.raises(RuntimeError, match="interrupted update"):
            rt.sweep()
    with patch.object(rt.model, "measure_with_energy", wraps=rt.model.measure_with_energy) as cached:
        actual = rt.measure()
    cached.assert_not_called()
    assert_meas_equal(actual, rt.model.measure(rt.state))

    rt = he3_runtime(L=4, R=2)
    e = cache_energy(rt)
    expected = rt.model.measure(rt.state)

    def fail_after_overwrite(state, output):
        output.copy_to_device(np.full(rt.R, 12345.0))
        raise RuntimeError("interrupted energy calculation")

    with patch.object(rt.model, "measure_energy", side_effect=fail_after_overwrite):
        with pytest.raises(RuntimeError, match="interrupted energy calculation"):
            rt.measure_energy(e)
    with patch.object(rt.model, "measure_with_energy", wraps=rt.model.measure_with_energy) as cached:
        actual = rt.measure()
    cached.assert_not_called()
    assert_meas_equal(actual, expected)


@pytest.mark.parametrize("name", ["xy", "ising", "kawamura"])
@pytest.mark.parametrize("L", [4, 6, 20])
def test_models_reuse_energy_and_preserve_ordering(name, L):
    """tests/test_energy_cache.py:343-400 including the sentinel energies."""
    from mcgb.core.runtime import Runtime
    from mcgb.device import to_device
    from mcgb.models.ising.model import IsingModel
    from mcgb.models.kawamura.model import KawamuraModel
    from mcgb.models.xy.model import XYModel
    rng = np.random.default_rng(215)
    model = {"xy": XYModel(J=1.3), "ising": IsingModel(J=0.9), "kawamura": KawamuraModel(J=1.1)}[name]
    rt = Runtime(model, L=L, temperatures=[0.4, 0.6, 0.8], threads=2, seed=216)
    if name == "xy":
        st = rng.uniform(-np.pi, np.pi, (3, L, L)).astype(np.float32)
    elif name == "ising":
        st = rng.choice([-1, 1], size=(3, L, L)).astype(np.int8)
    else:
        st = npref.random_kawamura(rng, 3, L)
    rt.state.copy_to_device(st)
    rt.invalidate_energy_cache()
    expected = model.measure(rt.state)
    e = cache_energy(rt)
    orig = e.copy_to_host()
    with patch.object(model, "measure_with_energy", wraps=model.measure_with_energy) as cached:
        actual = rt.measure()
    cached.assert_called_once()
    for k in expected:
        np.testing.assert_allclose(actual[k], expected[k], rtol=1e-12, atol=1e-10)
    np.testing.assert_array_equal(actual["energy"], orig)
    order = np.array([2, 0, 1], np.int32)
    mapping = to_device(order)
    ordered = rt.measure(temperature_indices=mapping)
    for k in actual:
        np.testing.assert_allclose(ordered[k][order], actual[k], rtol=1e-12, atol=1e-10)
    sentinel = np.array([12345., -6789., .125])
    e.copy_to_device(sentinel)
    reused = rt.measure(temperature_indices=mapping)
    np.testing.assert_array_equal(reused["energy"][order], sentinel)
    np.testing.assert_array_equal(e.copy_to_host(), sentinel)
    rt.sweep()
    with patch.object(model, "measure_with_energy", wraps=model.measure_with_energy) as cached:
        fresh = rt.measure()
    cached.assert_not_called()
    ref = model.measure(rt.state)
    for k in ref:
        np.testing.assert_array_equal(fresh[k], ref[k])


def test_simulation_schedule_both_models():
    """tests/test_simulation.py:137-165 (analysis/plots are outside this path)."""
    from mcgb.core.runtime import Runtime
    from mcgb.core.simulation import Simulation
    from mcgb.models.ising.model import IsingModel
    from mcgb.models.xy.model import XYModel
    for cls, temps in ((XYModel, [0.8, 1.0]), (IsingModel, [1.5, 2.0])):
        for L in (4, 8):
            rt = Runtime(cls(), L, temps, seed=42 + L)
            sim = Simulation(rt, thermalization_sweeps=4, measurement_sweeps=102, sample_interval=5)
            with patch.object(rt, "sweep", wraps=rt.sweep) as sweep:
                run = sim.run()
            assert sweep.call_count == 106
            np.testing.assert_array_equal(run["metadata"]["sample_sweeps"], np.arange(9, 105, 5))
            for v in run["samples"].values():
                assert isinstance(v, np.ndarray) and v.shape == (20, 2) and np.all(np.isfinite(v))
