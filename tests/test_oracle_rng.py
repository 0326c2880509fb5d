"""The oracle's xoroshiro128+ streams, pinned without the third-party package.

numba.cuda.random (Numba 0.68.0) is absent from this environment, and no
reference test pins raw RNG outputs.  The restatement is pinned instead by:
- published SplitMix64 known answers (the seeding step);
- the jump constant: Berlekamp-Massey recovers the engine's characteristic
  polynomial P from its output bits, and the constant must equal
  x^(2^64) mod P, i.e. a jump really advances 2^64 steps;
- structural properties of create_xoroshiro128p_states (stream k = k jumps).
"""

import numpy as np
import pytest

import gf2
import oracle


def test_splitmix64_published_vectors():
    # SplitMix64 first outputs for seeds 0 and 1234567 (published test values).
    assert oracle.splitmix64_first(0) == 0xE220A8397B1DCDAF
    assert oracle.splitmix64_first(1234567) == 6457827717110365317


def test_seed_fills_both_words_with_one_splitmix_output():
    s = oracle.rng_states(1, 42)
    z = oracle.splitmix64_first(42)
    assert int(s[0, 0]) == z and int(s[0, 1]) == z


@pytest.mark.parametrize("seed", [7, 2**63 + 5])
def test_jump_constant_is_x_to_2_64_mod_characteristic_polynomial(seed):
    st = oracle.rng_states(1, seed)[0].copy()
    bits = []
    for _ in range(400):
        bits.append(int(st[0]) & 1)
        oracle.rng_next(st)
    c, degree = gf2.berlekamp_massey(bits)
    assert degree == 128
    P = gf2.reciprocal(c, degree)
    jump = 0xBEAC0467EBA5FACB | (0xD86B048B86AA9922 << 64)
    assert gf2.x_pow_2k_mod(64, P) == jump


def test_jump_is_linear_polynomial_in_the_step_map():
    # jump(s) = sum_k c_k T^k s: check on a fresh state by explicit stepping.
    s0 = oracle.rng_states(1, 99)[0].copy()
    expected = s0.copy()
    oracle.rng_jump(expected)
    acc = np.zeros(2, dtype=np.uint64)
    st = s0.copy()
    jump = 0xBEAC0467EBA5FACB | (0xD86B048B86AA9922 << 64)
    for k in range(128):
        if (jump >> k) & 1:
            acc ^= st
        oracle.rng_next(st)
    np.testing.assert_array_equal(acc, expected)


def test_streams_are_successive_jumps_and_subsequence_offsets():
    a = oracle.rng_states(6, 1234)
    for k in range(1, 6):
        s = a[k - 1].copy()
        oracle.rng_jump(s)
        np.testing.assert_array_equal(s, a[k])
    b = oracle.rng_states(3, 1234, subsequence_start=3)
    np.testing.assert_array_equal(b, a[3:6])


def test_float32_uniform_is_rounded_float64_uniform():
    s = oracle.rng_states(2, 5)
    x = s[0].copy()
    y = s[0].copy()
    for _ in range(2000):
        f64 = oracle.uniform_f64(x)
        f32 = oracle.uniform_f32(y)
        assert np.float32(f64) == np.float32(f32)
        assert 0.0 <= f64 < 1.0 and 0.0 <= f32 <= 1.0


def test_next_output_is_sum_of_words_mod_2_64():
    s = oracle.rng_states(1, 11)[0].copy()
    expected = (int(s[0]) + int(s[1])) % 2**64
    assert oracle.rng_next(s) == expected
