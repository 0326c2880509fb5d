"""CUDA RNG streams and the Ising kernels against the oracle (bit-exact)."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    from mcgb import device, rng
    return device, rng


@pytest.mark.parametrize("n,seed,sub", [(1, 42, 0), (4097, 42, 0), (1000, 2**64 - 1, 0), (333, 7, 5)])
def test_device_jump_ahead_matches_sequential_host_jumps(dev, n, seed, sub):
    device, rng = dev
    states = rng.create_xoroshiro128p_states(n, seed, subsequence_start=sub)
    got = states.copy_to_host()
    ref = oracle.rng_states(n, seed, subsequence_start=sub)
    np.testing.assert_array_equal(got["s0"], ref[:, 0])
    np.testing.assert_array_equal(got["s1"], ref[:, 1])


def test_large_stream_index_matches_composed_jumps(dev):
    """Stream 2^20 + 3 from the device equals jumping stream 2^20 three times on the host."""
    device, rng = dev
    n = (1 << 20) + 4
    states = rng.create_xoroshiro128p_states(n, 2024).copy_to_host()
    base = np.array([states["s0"][1 << 20], states["s1"][1 << 20]], dtype=np.uint64)
    for _ in range(3):
        oracle.rng_jump(base)
    np.testing.assert_array_equal(base, [states["s0"][n - 1], states["s1"][n - 1]])


@pytest.mark.parametrize("kind", ["float32", "float64"])
def test_uniform_draws_match_oracle(dev, kind):
    device, rng = dev
    states = rng.create_xoroshiro128p_states(3, 77)
    got = rng.draw_uniforms(states, 2, 5000, kind)
    ref_state = oracle.rng_states(3, 77)[2].copy()
    draw = oracle.uniform_f32 if kind == "float32" else oracle.uniform_f64
    ref = np.array([draw(ref_state) for _ in range(5000)], dtype=got.dtype)
    np.testing.assert_array_equal(got, ref)


def _ising_runtime(L, temperatures, seed, init_seed):
    from mcgb.core.runtime import Runtime
    from mcgb.models.ising.model import IsingModel
    rt = Runtime(IsingModel(J=1.0), L, temperatures, seed=seed)
    spins = np.random.default_rng(init_seed).choice(np.array([-1, 1], dtype=np.int8), (len(temperatures), L, L))
    rt.state.copy_to_device(spins)
    return rt, spins


def cuda_ising_table(betas, J):
    """CUDA expf of the five Ising acceptance arguments per replica, (R, 5)."""
    from mcgb import _lib, device
    args = oracle.ising_exponent_arguments(betas, J)
    x = device.to_device(args)
    y = device.device_array(args.shape, np.float32)
    _lib.call("mcgb_expf", x.cptr, y.cptr, args.size, _lib.stream_handle())
    return y.copy_to_host()


def test_cuda_expf_within_documented_error_of_exact_exp(dev):
    """The reference's acceptance exponential is CUDA's float32 expf (its
    documented bound is 2 ulp).  Check that bound on the Ising arguments; the
    oracle then takes these CUDA values as inputs (orc_ising_sweeps_tab)."""
    betas = (1.0 / np.array([1.5, 2.269, 3.0, 2.0, 2.5, 0.6, 0.8, 1.0])).astype(np.float32)
    for J in (1.0, 1.37, 0.9):
        cuda = cuda_ising_table(betas, J)
        args = oracle.ising_exponent_arguments(betas, J)
        exact = np.exp(args.astype(np.float64))
        ulp = np.spacing(exact.astype(np.float32)).astype(np.float64)
        assert np.all(np.abs(cuda - exact) <= 2 * ulp)


@pytest.mark.parametrize("T", [1.5, 2.269, 3.0])
def test_ising_lattice_bit_exact_after_100_sweeps(T):
    """L=64, J=1, seeded uniform +-1 spins, seed 42+L: GPU lattice == oracle lattice."""
    L = 64
    rt, spins = _ising_runtime(L, [T], seed=42 + L, init_seed=42 + L)
    for _ in range(100):
        rt.sweep()
    got = rt.snapshot()
    ref = spins.copy()
    ref_rng = oracle.rng_states(L * L, 42 + L)
    betas = np.array([1 / T], np.float32)
    oracle.ising_sweeps_tab(ref, ref_rng, betas, cuda_ising_table(betas, 1.0), np.float32(1), 100)
    np.testing.assert_array_equal(got, ref)
    rs = rt.rng_states.copy_to_host()
    np.testing.assert_array_equal(rs["s0"], ref_rng[:, 0])
    np.testing.assert_array_equal(rs["s1"], ref_rng[:, 1])


def test_fused_three_phase_sweep_equals_four_colour_sweeps():
    L = 32
    a, spins = _ising_runtime(L, [1.5, 2.269, 3.0], seed=9, init_seed=10)
    b, _ = _ising_runtime(L, [1.5, 2.269, 3.0], seed=9, init_seed=10)
    for _ in range(25):
        a.sweep()
    b.model.sweep(b.state, b.rng_states, b.betas, n_sweeps=25)
    np.testing.assert_array_equal(a.snapshot(), b.snapshot())


def test_ising_updates_in_temperature_limits():
    """tests/test_simulation.py:108-135 (threads=2 forces a padded reference grid)."""
    from mcgb.core.runtime import Runtime
    from mcgb.models.ising.model import IsingModel
    import npref
    L = 6
    rt = Runtime(IsingModel(J=1.37), L, [1.0, 2.0], threads=2)
    expected = np.random.default_rng(19).choice(np.array([-1, 1], dtype=np.int8), (2, L, L))
    rt.state.copy_to_device(expected)
    rt.betas.copy_to_device(np.array([1e8, 0.0], dtype=np.float32))
    for color in range(4):
        npref.ising_beta_limit_colour(expected, color, hot=[False, True])
        rt.model.update_color(rt.state, rt.rng_states, rt.betas, color, rt.blocks_per_grid, rt.threads_per_block)
        np.testing.assert_array_equal(rt.snapshot(), expected)


def test_ising_measurements_exact():
    """tests/test_simulation.py:72-106."""
    from mcgb import device
    from mcgb.models.ising.model import IsingModel
    import npref
    model = IsingModel(J=1.37)
    L = 6
    cb = 1 - 2 * (np.indices((L, L)).sum(axis=0) % 2)
    spins = np.stack((np.ones((L, L)), -np.ones((L, L)), cb)).astype(np.int8)
    m = model.measure(device.to_device(spins))
    np.testing.assert_array_equal(m["energy"], float(model.J) * L**2 * np.array([-2.0, -2.0, 2.0]))
    np.testing.assert_array_equal(m["magnetization"], [L**2, -L**2, 0])
    rng = np.random.default_rng(18)
    for L in (4, 6, 32, 64):
        spins = rng.choice(np.array([-1, 1], dtype=np.int8), (3, L, L))
        m = model.measure(device.to_device(spins))
        ref = npref.ising(spins, model.J)
        assert m["energy"].dtype == np.float64
        np.testing.assert_array_equal(m["energy"], ref["energy"])
        np.testing.assert_array_equal(m["magnetization"], ref["magnetization"])
