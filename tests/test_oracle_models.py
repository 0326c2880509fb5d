"""The oracle against the reference tests' known answers and NumPy formulas.

Each case restates a reference test (file:line in the test docstrings) and
runs it on the CPU restatement, so the oracle is pinned before it checks the
CUDA kernels.
"""

import numpy as np
import pytest

import npref
import oracle

PRESSURE_CASES = (None, 0.0, 20.0, 34.0)


def he3_coefficients(pressure=None, reduced_temperature=1.0, betas=(-0.5, 1, 1, 1, -1)):
    from mcgb.models.he3.model import STRONG_COUPLING
    c = np.asarray(betas, dtype=np.float64)
    if pressure is not None:
        c = c + 0.5 * reduced_temperature * np.polynomial.polynomial.polyval(pressure / 34, STRONG_COUPLING)
    return c.astype(np.float32)


# ------------------------------------------------------------------ Ising

def test_ising_ordered_and_checkerboard_measurements():
    """tests/test_simulation.py:72-86."""
    J = np.float32(1.37)
    L = 6
    cb = 1 - 2 * (np.indices((L, L)).sum(axis=0) % 2)
    spins = np.stack((np.ones((L, L)), -np.ones((L, L)), cb)).astype(np.int8)
    out = oracle.ising_measure(spins, J)
    np.testing.assert_array_equal(out[0], float(J) * L**2 * np.array([-2.0, -2.0, 2.0]))
    np.testing.assert_array_equal(out[1], [L**2, -L**2, 0])


@pytest.mark.parametrize("L", [4, 6, 32, 64])
def test_ising_measure_matches_bond_count(L):
    """tests/test_simulation.py:88-106 (exact equality)."""
    J = np.float32(1.37)
    spins = np.random.default_rng(18).choice(np.array([-1, 1], dtype=np.int8), (3, L, L))
    out = oracle.ising_measure(spins, J)
    ref = npref.ising(spins, J)
    np.testing.assert_array_equal(out[0], ref["energy"])
    np.testing.assert_array_equal(out[1], ref["magnetization"])
    np.testing.assert_array_equal(oracle.ising_energy(spins, J), ref["energy"])


def test_ising_beta_limits_colour_by_colour():
    """tests/test_simulation.py:108-135: beta = 1e8 accepts only dE <= 0, beta = 0 all."""
    L = 6
    expected = np.random.default_rng(19).choice(np.array([-1, 1], dtype=np.int8), (2, L, L))
    spins = expected.copy()
    rng = oracle.rng_states(2 * L * L, 42)
    betas = np.array([1e8, 0.0], dtype=np.float32)
    for color in range(4):
        npref.ising_beta_limit_colour(expected, color, hot=[False, True])
        oracle.ising_update_color(spins, rng, betas, color, np.float32(1.37))
        np.testing.assert_array_equal(spins, expected)


def test_ising_sweeps_equal_colour_sequence_and_openmp():
    L, R = 16, 3
    spins = np.random.default_rng(3).choice(np.array([-1, 1], dtype=np.int8), (R, L, L))
    betas = (1 / np.array([1.5, 2.269, 3.0])).astype(np.float32)
    a, ra = spins.copy(), oracle.rng_states(R * L * L, 7)
    b, rb = spins.copy(), ra.copy()
    c, rc = spins.copy(), ra.copy()
    for _ in range(5):
        for color in range(4):
            oracle.ising_update_color(a, ra, betas, color, np.float32(1))
    oracle.ising_sweeps(b, rb, betas, np.float32(1), 5, n_threads=1)
    oracle.ising_sweeps(c, rc, betas, np.float32(1), 5, n_threads=3)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)
    np.testing.assert_array_equal(ra, rb)
    np.testing.assert_array_equal(ra, rc)


# ------------------------------------------------------------------ XY

def test_xy_ordered_measurements():
    """tests/test_simulation.py:25-41."""
    J = np.float32(1.37)
    out = oracle.xy_measure(np.zeros((2, 4, 4), np.float32), J)
    np.testing.assert_allclose(out[0], -2 * J * 16, atol=1e-12)
    np.testing.assert_allclose(out[1], 16, atol=1e-12)
    np.testing.assert_allclose(out[2:], [[0, 0], [16, 16], [0, 0]], atol=1e-12)


@pytest.mark.parametrize("L", [4, 6, 32])
def test_xy_measure_matches_complex_bonds(L):
    """tests/test_simulation.py:43-70."""
    J = np.float32(1.37)
    ang = np.random.default_rng(17).uniform(-np.pi, np.pi, (3, L, L)).astype(np.float32)
    out = oracle.xy_measure(ang, J)
    ref = npref.xy(ang, J)
    for c, name in enumerate(("energy", "mx", "my", "twist_cos_x", "twist_sin_x")):
        np.testing.assert_allclose(out[c], ref[name], rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(oracle.xy_energy(ang, J), ref["energy"], rtol=1e-12, atol=1e-10)


def test_xy_measure_ordering_and_cache():
    """tests/test_energy_cache.py:343-391: scatter by temperature, reuse supplied energies."""
    J = np.float32(1.3)
    ang = np.random.default_rng(215).uniform(-np.pi, np.pi, (3, 6, 6)).astype(np.float32)
    plain = oracle.xy_measure(ang, J)
    order = np.array([2, 0, 1], dtype=np.int32)
    ordered = oracle.xy_measure(ang, J, temperature_indices=order)
    np.testing.assert_array_equal(ordered[:, order], plain)
    sentinel = np.array([12345.0, -6789.0, 0.125])
    cached = oracle.xy_measure(ang, J, temperature_indices=order, cached=sentinel)
    np.testing.assert_array_equal(cached[0, order], sentinel)
    np.testing.assert_array_equal(cached[1:, order], plain[1:])


def test_xy_update_local_energy_change_is_metropolis_consistent():
    """At beta = 0 every proposal is accepted; the wrap keeps theta in [-pi, pi)."""
    L = 8
    ang = np.random.default_rng(1).uniform(-np.pi, np.pi, (2, L, L)).astype(np.float32)
    rng = oracle.rng_states(2 * L * L, 3)
    oracle.xy_sweeps(ang, rng, np.zeros(2, np.float32), np.float32(1), np.float32(1.5), 3)
    assert np.all(ang >= -np.pi) and np.all(ang < np.pi)
    g = np.random.default_rng(2).uniform(-np.pi, np.pi, (2, L, L)).astype(np.float32)
    oracle.xy_sweeps(g, oracle.rng_states(2 * L * L, 4), np.zeros(2, np.float32), np.float32(1),
                     np.float32(1.5), 3, sigmas=np.array([0.5, 3.0], np.float32))
    assert np.all(g >= -np.float32(np.pi)) and np.all(g < np.float32(np.pi))


# ------------------------------------------------------------------ Kawamura

def test_kawamura_ordered_observables():
    """tests/test_kawamura.py:62-71."""
    J = np.float32(1.37)
    st = np.zeros((2, 4, 4, 5), np.float32)
    st[..., 1] = 1
    st[..., 4] = 1
    out = oracle.kawamura_measure(st, J)
    expected = [-4 * float(J) * 16, 16, 16, 0, 2 * 16**2 / 9, 32, 0]
    for c, v in enumerate(expected):
        np.testing.assert_allclose(out[c], v, atol=1e-12)


@pytest.mark.parametrize("L", [4, 6, 20])
def test_kawamura_measure_matches_numpy(L):
    """tests/test_kawamura.py:79-94."""
    J = np.float32(1.37)
    st = npref.random_kawamura(np.random.default_rng(63), 3, L)
    out = oracle.kawamura_measure(st, J)
    ref = npref.kawamura(st, J)
    for c, name in enumerate(("energy", "chirality", "px", "py", "spin2", "twist_cos_x", "twist_sin_x")):
        np.testing.assert_allclose(out[c], ref[name], atol=1e-10, rtol=1e-12)
    np.testing.assert_allclose(oracle.kawamura_energy(st, J), ref["energy"], atol=1e-10)


def test_kawamura_local_energy_change_matches_total_hamiltonian():
    """tests/test_kawamura.py:96-115 (atol 3e-6, rtol 1e-5)."""
    J = np.float32(1.37)
    st = npref.random_kawamura(np.random.default_rng(63), 3, 6)
    old = npref.kawamura(st, J)["energy"]
    for field in ("phase", "chirality", "spin"):
        prop = st[:, 1, 2].copy()
        if field == "phase":
            prop[:, 0] += 0.7
        elif field == "chirality":
            prop[:, 1] *= -1
        else:
            prop[:, 2:] = np.array([0.6, 0, 0.8])
        diff = []
        for r in range(3):
            e0 = oracle.kawamura_local_energy(st, r, 1, 2, st[r, 1, 2], J)
            e1 = oracle.kawamura_local_energy(st, r, 1, 2, prop[r], J)
            diff.append(e1 - e0)
        changed = st.copy()
        changed[:, 1, 2] = prop
        np.testing.assert_allclose(diff, npref.kawamura(changed, J)["energy"] - old, atol=3e-6, rtol=1e-5)


def test_kawamura_hot_and_cold_limits():
    """tests/test_kawamura.py:128-143.

    At beta = 0 every tau flip is accepted (u < exp(0) = 1), so tau returns to
    +1 after an even number of sweeps and is -1 after an odd number.
    """
    L = 6
    st = np.zeros((2, L, L, 5), np.float32)
    st[..., 1] = 1
    st[..., 4] = 1
    rng = oracle.rng_states(2 * L * L, 42)
    oracle.kawamura_sweeps(st, rng, np.zeros(2, np.float32), np.float32(1), np.float32(1.5), 20)
    assert np.all(np.abs(st[..., 0]) <= np.pi + 1e-6)
    assert set(np.unique(st[..., 1])) == {1.0}
    odd = st.copy()
    oracle.kawamura_sweeps(odd, rng.copy(), np.zeros(2, np.float32), np.float32(1), np.float32(1.5), 1)
    assert set(np.unique(odd[..., 1])) == {-1.0}
    np.testing.assert_allclose(np.linalg.norm(st[..., 2:], axis=-1), 1, atol=2e-6)
    assert np.std(st[..., 0]) > 0.1 and np.std(st[..., 2:]) > 0.1
    cold = np.zeros((2, 4, 4, 5), np.float32)
    cold[..., 1] = 1
    cold[..., 4] = 1
    oracle.kawamura_sweeps(cold, oracle.rng_states(32, 42), np.full(2, 1e8, np.float32),
                           np.float32(1), np.float32(1.5), 4)
    np.testing.assert_allclose(oracle.kawamura_measure(cold, np.float32(1))[0], -64, atol=1e-5)


# ------------------------------------------------------------------ He3

def test_he3_ordered_state_closed_forms():
    """tests/test_he3.py:127-145."""
    K, betas = np.float32(1.3), np.array((-0.5, 1.0, 1.0, 1.0, -1.0), np.float32)
    B = float(betas[1] + betas[3] + betas[4])
    amp = np.float32(1 / np.sqrt(2 * B))
    st = np.zeros((2, 4, 4, 3, 2), np.complex64)
    st[..., 2, 0] = amp
    st[..., 2, 1] = 1j * amp
    n = float(np.sum(np.abs(st[0, 0, 0].astype(np.complex128))**2))
    out = oracle.he3_measure(st, betas, K)
    expected = [-2 * n * 16 + B * n**2 * 16, n * 16, n * 16, n * 16, 0, 0, 4 * float(K) * n * 16,
                0, 4 * float(K) * n * 16, 1]
    for c, v in enumerate(expected):
        np.testing.assert_allclose(out[c], v, atol=1e-6)


@pytest.mark.parametrize("L", [4, 6, 20])
def test_he3_measure_matches_numpy(L):
    """tests/test_he3.py:155-180 (per-site budgets in float32 eps)."""
    K = np.float32(0.73)
    betas = np.asarray((-0.4, 1.1, 0.8, 1.3, -0.7), np.float32)
    st = npref.random_he3(np.random.default_rng(253), (3, L, L, 3, 2))
    out = oracle.he3_measure(st, betas, K)
    ref = npref.he3(st, float(K), betas.astype(float))
    idx = {"energy": 0, "density": 1, "chirality": 2, "phase_real": 3, "phase_imag": 4, "spin_alignment": 9}
    for name, c in idx.items():
        budget = (8 if name == "energy" else 2) * np.finfo(np.float32).eps
        np.testing.assert_allclose(out[c] / L**2, ref[name] / L**2, atol=budget, rtol=0, err_msg=name)
    np.testing.assert_array_equal(oracle.he3_energy(st, betas, K), out[0])


def test_he3_helicity_matches_twisted_hamiltonian_derivatives():
    """tests/test_he3.py:182-197."""
    K = np.float32(0.73)
    betas = np.asarray((-0.4, 1.1, 0.8, 1.3, -0.7), np.float32)
    st = npref.random_he3(np.random.default_rng(253), (3, 4, 4, 3, 2))
    out = oracle.he3_measure(st, betas, K)
    h = 2e-4
    e = npref.he3_energy(st, float(K), betas.astype(float))
    for axis, (ci, ki) in enumerate(((5, 6), (7, 8))):
        tw = np.zeros(2)
        tw[axis] = h
        plus = npref.he3_energy(st, float(K), betas.astype(float), tw)
        minus = npref.he3_energy(st, float(K), betas.astype(float), -tw)
        np.testing.assert_allclose(out[ci], (plus - minus) / (2 * h), atol=2e-6, rtol=1e-7)
        np.testing.assert_allclose(out[ki], (plus - 2 * e + minus) / h**2, atol=2e-5, rtol=1e-6)


def test_he3_spin_alignment_normalisation():
    """tests/test_he3.py:238-251."""
    st = np.zeros((5, 4, 4, 3, 2), np.complex64)
    orb = np.array([1, 1j], np.complex64) / np.sqrt(2)
    st[0, ..., 2, :] = orb
    st[1, ..., 0, :] = orb
    st[2] = np.ones((3, 1)) * orb / np.sqrt(3)
    st[3, :2, :, 2, :] = np.sqrt(3) * orb
    st[3, 2:, :, 0, :] = orb
    out = oracle.he3_measure(st, np.array((-0.5, 1, 1, 1, -1), np.float32), np.float32(1), g_d=0.001)
    np.testing.assert_allclose(out[9], [1, -0.5, 0, 0.625, 0], atol=1e-7, rtol=0)


@pytest.mark.parametrize("L", [4, 6, 20])
@pytest.mark.parametrize("pressure", PRESSURE_CASES)
def test_he3_direct_difference_matches_full_change(L, pressure):
    """tests/test_he3_energy_difference.py:137-160, 305-322 with its error budgets."""
    K = np.float32(0.73)
    coeff = he3_coefficients(pressure)
    rng = np.random.default_rng(20261027)
    pos = np.array([(0, 0), (0, L - 1), (L - 1, 0), (L - 1, L - 1), (0, L // 2), (L // 2, 0),
                    (L - 1, L // 2), (L // 2, L - 1), (1, 1), (1, 2), (2, 1), (2, 2)], np.int32)
    st = npref.random_he3(rng, (len(pos), L, L, 3, 2))
    old = np.stack([st[r, i, j] for r, (i, j) in enumerate(pos)])
    re = rng.uniform(-0.15, 0.15, size=old.shape).astype(np.float32)
    im = rng.uniform(-0.15, 0.15, size=old.shape).astype(np.float32)
    prop = np.empty_like(old)
    prop.real = old.real + re
    prop.imag = old.imag + im
    dg = np.array([oracle.he3_gradient_difference(st, r, i, j, prop[r]) for r, (i, j) in enumerate(pos)])
    dv = np.array([oracle.he3_potential(prop[r], coeff) - oracle.he3_potential(old[r], coeff)
                   for r in range(len(pos))], dtype=np.float64)
    changed = st.copy()
    for r, (i, j) in enumerate(pos):
        changed[r, i, j] = prop[r]
    ov, og = npref.he3_energy_parts(st, coeff)
    nv, ng = npref.he3_energy_parts(changed, coeff)
    np.testing.assert_allclose(dg, ng - og, rtol=3e-6, atol=6e-6)
    _, old_scale = npref.he3_potential(old, coeff)
    _, new_scale = npref.he3_potential(prop, coeff)
    eps = np.finfo(np.float32).eps
    np.testing.assert_array_less(np.abs(dv - (nv - ov)), 8 * eps * np.maximum(1, old_scale + new_scale))


def test_he3_hot_moves_and_cold_minimum():
    """tests/test_he3.py:352-366."""
    coeff = np.array((-0.5, 1, 1, 1, -1), np.float32)
    amp = np.float32(1 / np.sqrt(2 * 1.0))
    st = np.zeros((2, 6, 6, 3, 2), np.complex64)
    st[..., 2, 0] = amp
    st[..., 2, 1] = 1j * amp
    init = st.copy()
    oracle.he3_sweeps(st, oracle.rng_states(72, 42), np.zeros(2, np.float32), coeff, np.float32(1),
                      np.float32(0.15), np.float32(0), 10)
    assert np.isfinite(st).all() and np.std(st - init) > 0.03
    cold = np.zeros((2, 4, 4, 3, 2), np.complex64)
    cold[..., 2, 0] = amp
    cold[..., 2, 1] = 1j * amp
    e0 = oracle.he3_energy(cold, coeff, np.float32(1))
    oracle.he3_sweeps(cold, oracle.rng_states(32, 42), np.full(2, 1e8, np.float32), coeff, np.float32(1),
                      np.float32(0.15), np.float32(0), 4)
    np.testing.assert_allclose(oracle.he3_energy(cold, coeff, np.float32(1)), e0, atol=1e-5)


def test_he3_gaussian_sampler_counts_and_finiteness():
    """models/he3/gaussian_fast.py:91-119: every visit counted, no nonfinite ratios."""
    coeff = he3_coefficients(20.0)
    st = npref.random_he3(np.random.default_rng(5), (3, 6, 6, 3, 2))
    counts = oracle.he3_sweeps(st, oracle.rng_states(108, 227), (1 / np.array([0.3, 0.4, 0.6])).astype(np.float32),
                               coeff, np.float32(1), np.float32(0.15), np.float32(0), 4, gaussian=True,
                               rho=np.float32(-0.9), mass=np.float32(0))
    assert counts[0].sum() == 4 * 3 * 36
    assert counts[2].sum() == 0
    assert 0 < counts[1].sum() < counts[0].sum()
    assert np.isfinite(st).all()
