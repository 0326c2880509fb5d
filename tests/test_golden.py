"""The oracle against the committed golden fixtures (tests/golden/,
written by tests/golden/make_golden.py).

The RNG fixture comes from a pure-Python restatement of xoroshiro128+ and
its seeding, independent of the C oracle, so agreement pins both.  The sweep
and exchange fixtures pin the oracle's behaviour: any change to its
arithmetic or draw order shows up here before it reaches a GPU comparison.
"""

import json
from pathlib import Path

import numpy as np
import pytest

import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"


def rng_cases():
    return json.loads((GOLDEN / "rng_streams.json").read_text())["cases"]


@pytest.fixture(scope="module")
def sweeps():
    return dict(np.load(GOLDEN / "sweeps.npz"))


@pytest.mark.parametrize("case", rng_cases(), ids=lambda c: f"seed{c['seed']}-stream{c['stream']}")
def test_oracle_streams_match_the_independent_restatement(case):
    states = oracle.rng_states(case["stream"] + 1, case["seed"])
    st = states[case["stream"]].copy()
    assert [f"{v:016x}" for v in st] == case["state"]
    raw = [oracle.rng_next(st) for _ in range(4)]
    assert [f"{v:016x}" for v in raw] == case["raw"]
    st = states[case["stream"]].copy()
    assert [oracle.uniform_f64(st).hex() for _ in range(4)] == case["uniform_f64"]
    st = states[case["stream"]].copy()
    bits = [f"{int(np.float32(oracle.uniform_f32(st)).view(np.uint32)):08x}" for _ in range(4)]
    assert bits == case["uniform_f32_bits"]


def test_ising_fixture_table_is_within_cuda_expf_error_of_exp(sweeps):
    """The captured CUDA expf values lie within 2 ulp of the exact exponential."""
    table = sweeps["ising_table"]
    args = oracle.ising_exponent_arguments(sweeps["ising_betas"], 1.0)
    exact = np.exp(args.astype(np.float64))
    ulp = np.spacing(table.astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(table - exact) <= 2 * ulp)


def test_ising_fixture(sweeps):
    s = sweeps
    state, rng = s["ising_in"].copy(), oracle.rng_states(s["ising_in"].size, int(s["ising_seed"]))
    oracle.ising_sweeps_tab(state, rng, s["ising_betas"], s["ising_table"], np.float32(1), int(s["ising_sweeps"]))
    np.testing.assert_array_equal(state, s["ising_out"])
    np.testing.assert_array_equal(rng, s["ising_rng_out"])
    np.testing.assert_array_equal(oracle.ising_measure(state, np.float32(1)), s["ising_measure"])


@pytest.mark.parametrize("name", ["xy", "xyg"])
def test_xy_fixtures(sweeps, name):
    s = sweeps
    state = s[f"{name}_in"].copy()
    rng = oracle.rng_states(state.size, int(s[f"{name}_seed"]))
    oracle.xy_sweeps(state, rng, s[f"{name}_betas"], np.float32(1), np.float32(1.5), int(s[f"{name}_sweeps"]),
                     sigmas=s["xyg_sigmas"] if name == "xyg" else None)
    np.testing.assert_array_equal(state, s[f"{name}_out"])
    np.testing.assert_array_equal(rng, s[f"{name}_rng_out"])
    np.testing.assert_array_equal(oracle.xy_measure(state, np.float32(1)), s[f"{name}_measure"])


def test_kawamura_fixture(sweeps):
    s = sweeps
    state = s["kaw_in"].copy()
    rng = oracle.rng_states(state.shape[0] * state.shape[1] ** 2, int(s["kaw_seed"]))
    oracle.kawamura_sweeps(state, rng, s["kaw_betas"], np.float32(1), np.float32(1.5), int(s["kaw_sweeps"]))
    np.testing.assert_array_equal(state, s["kaw_out"])
    np.testing.assert_array_equal(rng, s["kaw_rng_out"])
    np.testing.assert_array_equal(oracle.kawamura_measure(state, np.float32(1)), s["kaw_measure"])


def test_kawamura_gaussian_fixture(sweeps):
    s = sweeps
    state = s["kaw_in"].copy()
    rng = oracle.rng_states(state.shape[0] * state.shape[1] ** 2, int(s["kaw_seed"]))
    oracle.kawamura_sweeps_gauss(state, rng, s["kaw_betas"], s["kawg_sigmas"], np.float32(1), int(s["kaw_sweeps"]))
    np.testing.assert_array_equal(state, s["kawg_out"])
    np.testing.assert_array_equal(rng, s["kawg_rng_out"])


@pytest.mark.parametrize("name", ["he3", "he3g"])
def test_he3_fixtures(sweeps, name):
    s = sweeps
    state = s[f"{name}_in"].copy()
    rng = oracle.rng_states(state.shape[0] * state.shape[1] ** 2, int(s[f"{name}_seed"]))
    counts = oracle.he3_sweeps(state, rng, s[f"{name}_betas"], s["he3_coefficients"], np.float32(1),
                               np.float32(0.15), np.float32(0), int(s[f"{name}_sweeps"]), gaussian=name == "he3g",
                               rho=np.float32(-0.9), mass=np.float32(0))
    np.testing.assert_array_equal(state, s[f"{name}_out"])
    np.testing.assert_array_equal(rng, s[f"{name}_rng_out"])
    np.testing.assert_array_equal(oracle.he3_measure(state, s["he3_coefficients"], np.float32(1)),
                                  s[f"{name}_measure"])
    if name == "he3g":
        np.testing.assert_array_equal(counts, s["he3g_counts"])


def test_exchange_fixture():
    p = dict(np.load(GOLDEN / "pt.npz"))
    R = len(p["betas_in"])
    b, w2t, t2w = p["betas_in"].copy(), np.arange(R, dtype=np.int32), np.arange(R, dtype=np.int32)
    rng, counts, trips = oracle.rng_states(R - 1, int(p["seed"])), np.zeros((3, R - 1), np.int64), \
        oracle.pt_initial_trips(R)
    for k, e in enumerate(p["energies"]):
        oracle.pt_exchange(np.ascontiguousarray(e), b, w2t, t2w, rng, counts, trips, k & 1, 10 * (k + 1))
        for name, v in (("w2t", w2t), ("t2w", t2w), ("betas", b), ("counts", counts), ("trips", trips)):
            np.testing.assert_array_equal(v, p[name][k], err_msg=f"{name} after round {k}")
    # The fixture exercises both outcomes and completes at least one round trip.
    assert 0 < p["counts"][-1][1].sum() < p["counts"][-1][0].sum()
    assert p["trips"][-1][3].sum() > 0
