"""The block-jackknife helpers of the statistical parity tests, on CPU."""

import numpy as np
import pytest

import stats


def test_jackknife_of_a_mean_is_the_standard_error_of_block_means():
    x = np.random.default_rng(3).normal(size=(1000, 4))
    value, error = stats.jackknife({"x": x}, lambda m: m["x"], 50)
    blocks = x.reshape(20, 50, 4).mean(axis=1)
    np.testing.assert_allclose(value, x.mean(axis=0), rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(error, blocks.std(axis=0, ddof=1) / np.sqrt(20), rtol=1e-10)


def test_jackknife_propagates_a_nonlinear_estimator():
    rng = np.random.default_rng(4)
    x = 2.0 + 0.1 * rng.normal(size=20000)
    value, error = stats.jackknife({"x": x}, lambda m: m["x"] ** 2, 100)
    # delta method: d(x^2) = 2 x dx
    assert value == pytest.approx(x.mean() ** 2)
    assert error == pytest.approx(2 * 2.0 * 0.1 / np.sqrt(len(x)), rel=0.35)


def test_incomplete_blocks_are_dropped_and_two_are_required():
    assert stats.blocks_of(np.arange(10.0), 4).tolist() == [1.5, 5.5]
    with pytest.raises(ValueError):
        stats.blocks_of(np.arange(7.0), 4)


def test_xy_estimators_on_an_ordered_chain():
    n, L, T = 400, 4, np.array([0.5, 1.0])
    N = L * L
    samples = {"energy": np.full((n, 2), -2.0 * N), "mx": np.full((n, 2), float(N)), "my": np.zeros((n, 2)),
               "twist_cos_x": np.full((n, 2), float(N)), "twist_sin_x": np.zeros((n, 2))}
    obs = stats.xy_observables(samples, L, T, block_size=100)
    np.testing.assert_allclose(obs["energy"][0], -2.0)
    np.testing.assert_allclose(obs["binder"][0], 0.5)
    np.testing.assert_allclose(obs["helicity"][0], 1.0)
    np.testing.assert_allclose(obs["energy"][1], 0.0)


def test_compare_flags_only_differences_beyond_the_bound():
    a = {"e": (np.array([1.0, 2.0]), np.array([0.1, 0.1]))}
    b = {"e": (np.array([1.2, 3.0]), np.array([0.1, 0.1]))}
    bad = stats.compare(a, b, 3.0)
    assert [(name, k) for name, k, *_ in bad] == [("e", 1)]


def test_family_bound_reproduces_the_single_test_rate():
    assert stats.family_bound(1) == pytest.approx(3.0, abs=1e-9)
    # 18 comparisons at a 0.27 % family-wise rate: 3.79 sigma each.
    assert stats.family_bound(18) == pytest.approx(3.791, abs=0.001)
    assert stats.family_bound(28) > stats.family_bound(18)


def test_linear_crossings_follow_the_reference_rules():
    T = np.array([1.0, 2.0, 3.0, 4.0])
    assert stats.linear_crossings(T, [0, 1, 2, 3], [3, 2, 1, 0]) == [2.5]
    assert stats.linear_crossings(T, [1, 2, 2, 4], [0, 2, 3, 3]) == [2.0, 3.5]
    assert stats.linear_crossings(T, [1, 1, 2, 3], [1, 1, 0, 0]) == []   # an interval of roots
    assert stats.linear_crossings(T, [1, 2, 3, 4], [0, 0, 0, 0]) == []


def test_binder_crossing_recovers_a_planted_crossing():
    # m2 = 1 + s z^2 (z normal) has Binder value 1 - (1 + 2s + 3s^2) / (2 (1 + s)^2),
    # monotonic in s; s_a(T) and s_b(T) are equal at T = 1.5 only.
    r = np.random.default_rng(3)
    T = np.linspace(1.0, 2.0, 11)
    n = 20000

    def fake(slope):
        scale = np.exp(slope * (T - 1.5))
        return {"m2": 1 + scale * r.normal(size=(n, T.size)) ** 2}
    binder = (lambda m: 1 - m["m4"] / (2 * m["m2"] ** 2))
    got = stats.binder_crossing(fake(1.0), fake(-1.0), T, binder, block_size=1000)
    assert got is not None
    value, err = got
    assert 0 < err < 0.05 and abs(value - 1.5) < 4 * err
