"""Simulation's graph replay against its step-by-step loop.

Simulation.run() replays the schedule of a built-in model as captured CUDA
graphs with a device clock for the exchanges and device rings for samples
and walker history (mcgb/core/schedule.py).  It launches the kernels of the
step-by-step loop in the same order, so everything must be bit-identical to
``replay = False``: samples, sample sweeps, every diagnostic (maps, swap and
round-trip counters, walker history), final state, RNG streams, betas, the
exchange energies, the runtime's energy cache, and the He3 Gaussian
counters -- over consecutive runs, for every model, with and without PT.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def build(kind, R, L, seed, pt_kw=None, runtime_kw=None):
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    T = np.geomspace(0.7, 1.2, R) if kind not in ("ising", "he3", "he3g") else (
        np.geomspace(1.8, 3.0, R) if kind == "ising" else np.geomspace(0.33, 0.47, R))
    r = np.random.default_rng(seed)
    cls = Runtime
    if kind == "ising":
        from mcgb.models.ising.model import IsingModel
        model, init = IsingModel(), r.choice(np.array([-1, 1], np.int8), (R, L, L))
    elif kind in ("xy", "xyg"):
        from mcgb.device import to_device
        from mcgb.models.xy.model import XYModel
        sig = to_device(np.linspace(0.8, 1.6, R).astype(np.float32)) if kind == "xyg" else None
        model = XYModel(proposal="gaussian" if kind == "xyg" else "uniform", sigmas=sig)
        init = r.uniform(-np.pi, np.pi, (R, L, L)).astype(np.float32)
    elif kind == "kawamura":
        from mcgb.models.kawamura.model import KawamuraModel
        model = KawamuraModel()
        init = np.zeros((R, L, L, 5), np.float32)
        init[..., 0] = r.uniform(-np.pi, np.pi, (R, L, L))
        init[..., 1] = r.choice([-1.0, 1.0], (R, L, L))
        d = r.normal(size=(R, L, L, 3))
        init[..., 2:] = d / np.linalg.norm(d, axis=-1, keepdims=True)
    else:
        from mcgb.models.he3.model import He3Model
        model = He3Model(pressure=20, g_d=0.001) if kind == "he3" else He3Model()
        a = 0.3 * np.sqrt(2)
        init = (r.uniform(-a, a, (R, L, L, 3, 2)) + 1j * r.uniform(-a, a, (R, L, L, 3, 2))).astype(np.complex64)
        if kind == "he3g":
            from mcgb.models.he3.sampling import He3GaussianRuntime
            cls = He3GaussianRuntime
    rt = cls(model, L, T, seed=seed, **(runtime_kw or {}))
    rt.state.copy_to_device(init)
    if pt_kw is None:
        return rt, rt
    return rt, ParallelTempering(rt, **pt_kw)


def run_pair(kind, R, L, seed, runs, pt_kw=None):
    from mcgb.core.simulation import Simulation
    results = []
    for replay in (True, False):
        rt, top = build(kind, R, L, seed, pt_kw)
        outs = []
        for therm, meas, every in runs:
            sim = Simulation(top, thermalization_sweeps=therm, measurement_sweeps=meas, sample_interval=every)
            sim.replay = replay
            outs.append(sim.run())
        results.append((rt, top, outs))
    return results


def assert_same(a, b, path="result"):
    if isinstance(a, dict):
        assert a.keys() == b.keys(), path
        for k in a:
            assert_same(a[k], b[k], f"{path}.{k}")
    elif a is None or isinstance(a, (str, int, float, np.floating, np.integer)):
        assert a == b, path
    else:
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b), err_msg=path)


def compare(results):
    (rt_a, top_a, outs_a), (rt_b, top_b, outs_b) = results
    for a, b in zip(outs_a, outs_b):
        assert_same(a, b)
    np.testing.assert_array_equal(rt_a.snapshot(), rt_b.snapshot())
    ra, rb = rt_a.rng_states.copy_to_host(), rt_b.rng_states.copy_to_host()
    np.testing.assert_array_equal(ra["s0"], rb["s0"])
    np.testing.assert_array_equal(ra["s1"], rb["s1"])
    np.testing.assert_array_equal(rt_a.betas.copy_to_host(), rt_b.betas.copy_to_host())
    # The energy cache: valid after a run that ended with an exchange, and
    # the measurement it serves is the same.
    assert (rt_a._energy.current() is None) == (rt_b._energy.current() is None)
    assert_same(top_a.measure(), top_b.measure())
    if top_a is not rt_a:
        np.testing.assert_array_equal(top_a.energies.copy_to_host(), top_b.energies.copy_to_host())
        assert (top_a.sweeps, top_a.exchange_rounds, top_a._parity) == (top_b.sweeps, top_b.exchange_rounds,
                                                                      top_b._parity)
        assert_same(top_a.diagnostics(), top_b.diagnostics())
    if hasattr(rt_a, "gaussian"):
        np.testing.assert_array_equal(rt_a.gaussian.counts.copy_to_host(), rt_b.gaussian.counts.copy_to_host())
        assert_same(rt_a.sampling_diagnostics(), rt_b.sampling_diagnostics())


@pytest.mark.parametrize("kind", ["ising", "xy", "xyg", "kawamura", "he3", "he3g"])
def test_replay_equals_step_by_step_with_pt(kind):
    runs = [(7, 40, 2), (3, 25, 5)]
    compare(run_pair(kind, 5, 8 if kind.startswith("he3") else 16, 11,
                     runs, pt_kw=dict(exchange_interval=3, tracked_walkers=[0, 4], history_stride=2)))


@pytest.mark.parametrize("kind", ["ising", "xy", "he3g"])
def test_replay_equals_step_by_step_without_pt(kind):
    compare(run_pair(kind, 3, 16, 12, [(5, 30, 3), (0, 7, 7)]))


def test_replay_captures_graphs_on_long_periodic_runs():
    """1,300 sweeps at interval 10 and sample interval 10: chunks of 64
    segments repeat, so they are captured and replayed; still bit-identical,
    with two-walker ladders (parity always 0)."""
    from unittest.mock import patch
    import torch
    captured = []
    orig = torch.cuda.CUDAGraph.replay

    def counting(self):
        captured.append(self)
        return orig(self)
    with patch.object(torch.cuda.CUDAGraph, "replay", counting):
        results = run_pair("xy", 2, 16, 13, [(20, 1280, 10)], pt_kw=dict(exchange_interval=10))
    assert len(captured) >= 2
    compare(results)


def test_custom_model_subclass_runs_step_by_step():
    """A user subclass of a built-in model keeps its own Python update_color:
    the schedule runs step by step through it (no replay)."""
    from mcgb.core.runtime import Runtime
    from mcgb.core.schedule import GraphReplay
    from mcgb.core.simulation import Simulation
    from mcgb.models.ising.model import IsingModel

    class Counting(IsingModel):
        calls = 0

        def update_color(self, *args, **kw):
            Counting.calls += 1
            return super().update_color(*args, **kw)
    rt = Runtime(Counting(), 8, [2.0, 2.5], seed=3)
    assert not GraphReplay.supports(rt)
    Simulation(rt, thermalization_sweeps=2, measurement_sweeps=4, sample_interval=2).run()
    assert Counting.calls == 4 * 6
