"""The CUDA path against the committed golden fixtures (tests/golden/).

Everything runs through the drop-in classes (Runtime, He3GaussianRuntime,
the model plugins) and the C ABI, from the fixture's inputs.  RNG streams,
Ising lattices, exchange maps and counters must match bit for bit;
continuous states within float32 rounding (1e-5), where an accept/reject
decision may differ only for a uniform within rounding of the acceptance
probability (at most 0.1 % of sites); measurement channels of the fixture's
final states to 1e-9 relative (float64 sums in another order; 1e-6 for
He3, whose per-site terms are float32).
"""

import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
STATE_TOL = 1e-5
MAX_FLIP_FRACTION = 1e-3


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(GOLDEN / "sweeps.npz"))


def _states_close(got, ref, site_axes):
    diff = np.abs(got.astype(np.complex128) - ref.astype(np.complex128))
    if site_axes:
        diff = diff.max(axis=site_axes)
    bad = diff > STATE_TOL
    assert bad.mean() <= MAX_FLIP_FRACTION, f"{bad.sum()} of {bad.size} sites differ"


def _rng_equal(device_states, ref):
    got = device_states.copy_to_host()
    np.testing.assert_array_equal(got["s0"], ref[:, 0])
    np.testing.assert_array_equal(got["s1"], ref[:, 1])


def _measure_close(m, names, ref, rtol=1e-9):
    for k, name in enumerate(names):
        np.testing.assert_allclose(m[name], ref[k], rtol=rtol, atol=rtol, err_msg=name)


def test_device_streams_match_golden_vectors():
    from mcgb import rng
    for case in json.loads((GOLDEN / "rng_streams.json").read_text())["cases"]:
        states = rng.create_xoroshiro128p_states(case["stream"] + 1, case["seed"])
        got = states.copy_to_host()[case["stream"]]
        assert [f"{int(got['s0']):016x}", f"{int(got['s1']):016x}"] == case["state"], case
        u64 = rng.draw_uniforms(states, case["stream"], 4, "float64")
        assert [float(x).hex() for x in u64] == case["uniform_f64"], case
        states = rng.create_xoroshiro128p_states(case["stream"] + 1, case["seed"])
        u32 = rng.draw_uniforms(states, case["stream"], 4, "float32")
        assert [f"{int(x.view(np.uint32)):08x}" for x in u32] == case["uniform_f32_bits"], case


def _runtime(fx, name, model, cls=None):
    from mcgb.core.runtime import Runtime
    cls = cls or Runtime
    state = fx[f"{name}_in"]
    R, L = state.shape[0], state.shape[1]
    rt = cls(model, L, list(1.0 / fx[f"{name}_betas"].astype(np.float64)), seed=int(fx[f"{name}_seed"]))
    rt.betas.copy_to_device(fx[f"{name}_betas"])
    rt.state.copy_to_device(state)
    for _ in range(int(fx[f"{name}_sweeps"])):
        rt.sweep()
    return rt


def test_ising_golden_sweeps_bit_exact(fx):
    from mcgb import _lib, device
    from mcgb.models.ising.model import MEASUREMENT_NAMES, IsingModel
    # The fixture's acceptance table must be the table CUDA's expf gives here.
    k = np.array([-8, -4, 0, 4, 8], np.float32)
    args = (-fx["ising_betas"][:, None] * k[None, :]).astype(np.float32)
    x, y = device.to_device(args), device.device_array(args.shape, np.float32)
    _lib.call("mcgb_expf", x.cptr, y.cptr, args.size, _lib.stream_handle())
    np.testing.assert_array_equal(y.copy_to_host(), fx["ising_table"])
    rt = _runtime(fx, "ising", IsingModel(J=1.0))
    np.testing.assert_array_equal(rt.snapshot(), fx["ising_out"])
    _rng_equal(rt.rng_states, fx["ising_rng_out"])
    m = IsingModel(J=1.0).measure(device.to_device(fx["ising_out"]))
    for i, name in enumerate(MEASUREMENT_NAMES):
        np.testing.assert_array_equal(m[name], fx["ising_measure"][i])


@pytest.mark.parametrize("name", ["xy", "xyg"])
def test_xy_golden_sweeps(fx, name):
    from mcgb import device
    from mcgb.models.xy.model import MEASUREMENT_NAMES, XYModel
    model = XYModel(J=1.0, proposal="gaussian" if name == "xyg" else "uniform",
                    sigmas=device.to_device(fx["xyg_sigmas"]) if name == "xyg" else None)
    rt = _runtime(fx, name, model)
    _rng_equal(rt.rng_states, fx[f"{name}_rng_out"])
    _states_close(rt.snapshot(), fx[f"{name}_out"], None)
    _measure_close(XYModel(J=1.0).measure(device.to_device(fx[f"{name}_out"])), MEASUREMENT_NAMES,
                   fx[f"{name}_measure"])


def test_kawamura_golden_sweeps(fx):
    from mcgb import device
    from mcgb.models.kawamura.model import MEASUREMENT_NAMES, KawamuraModel
    rt = _runtime(fx, "kaw", KawamuraModel(J=1.0, delta=1.5))
    _rng_equal(rt.rng_states, fx["kaw_rng_out"])
    _states_close(rt.snapshot(), fx["kaw_out"], (-1,))
    _measure_close(KawamuraModel(J=1.0).measure(device.to_device(fx["kaw_out"])), MEASUREMENT_NAMES,
                   fx["kaw_measure"])


def test_kawamura_gaussian_golden_sweeps(fx):
    from mcgb.batch import LadderBatch
    from mcgb.models.kawamura.model import KawamuraModel
    init = fx["kaw_in"]
    T = 1.0 / fx["kaw_betas"].astype(np.float64)
    b = LadderBatch(KawamuraModel(), [(init.shape[1], T)], seeds=[int(fx["kaw_seed"])], exchange_interval=None,
                    proposal="gaussian", initial_states=[init])
    b.betas.copy_to_device(fx["kaw_betas"])
    b.sigma_t.copy_to_device(fx["kawg_sigmas"])
    b.run(int(fx["kaw_sweeps"]))
    rng = b.ladder_rng(0)
    np.testing.assert_array_equal(rng, fx["kawg_rng_out"])
    _states_close(b.ladder_state(0), fx["kawg_out"], (-1,))


@pytest.mark.parametrize("name", ["he3", "he3g"])
def test_he3_golden_sweeps(fx, name):
    from mcgb import device
    from mcgb.models.he3.model import MEASUREMENT_NAMES, He3Model
    from mcgb.models.he3.sampling import He3GaussianRuntime
    model = He3Model()
    np.testing.assert_array_equal(model.coefficients(), fx["he3_coefficients"])
    rt = _runtime(fx, name, model, cls=He3GaussianRuntime if name == "he3g" else None)
    _rng_equal(rt.rng_states, fx[f"{name}_rng_out"])
    _states_close(rt.snapshot(), fx[f"{name}_out"], (-2, -1))
    # He3 local terms are float32 (the reference's arithmetic); the GPU may
    # contract them into fused multiply-adds, so per-site values differ by
    # float32 rounding and the sums by ~1e-8 relative.
    _measure_close(He3Model().measure(device.to_device(fx[f"{name}_out"])), MEASUREMENT_NAMES,
                   fx[f"{name}_measure"], rtol=1e-6)
    if name == "he3g":
        d = rt.sampling_diagnostics()
        counts = fx["he3g_counts"]
        assert sum(d["attempts"]) == counts[0].sum()
        assert abs(sum(d["accepted"]) - counts[1].sum()) <= MAX_FLIP_FRACTION * counts[0].sum() + 1


def test_exchange_golden_rounds():
    from mcgb import _lib, device
    from mcgb.rng import create_xoroshiro128p_states
    p = dict(np.load(GOLDEN / "pt.npz"))
    R = len(p["betas_in"])
    betas = device.to_device(p["betas_in"])
    w2t = device.to_device(np.arange(R, dtype=np.int32))
    t2w = device.to_device(np.arange(R, dtype=np.int32))
    rng = create_xoroshiro128p_states(R - 1, int(p["seed"]))
    counts = device.device_zeros((3, R - 1), np.int64)
    trips = np.zeros((5, R), np.int64)
    trips[0] = -1
    trips[2] = -1
    trips[0, 0], trips[0, -1] = 0, R - 1
    trips[2, [0, -1]] = 0
    trips = device.to_device(trips)
    energies = device.device_zeros(R, np.float64)
    for k, e in enumerate(p["energies"]):
        energies.copy_to_device(np.ascontiguousarray(e))
        _lib.call("mcgb_pt_exchange", energies.cptr, betas.cptr, w2t.cptr, t2w.cptr, rng.cptr, counts.cptr,
                  trips.cptr, R, k & 1, 10 * (k + 1), _lib.stream_handle())
        for name, v in (("w2t", w2t), ("t2w", t2w), ("betas", betas), ("counts", counts), ("trips", trips)):
            np.testing.assert_array_equal(v.copy_to_host(), p[name][k], err_msg=f"{name} after round {k}")
