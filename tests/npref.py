"""Independent float64 NumPy formulas for the observables and Hamiltonians.

These restate the reference tests' NumPy checks (tests/test_simulation.py:53-65,
tests/test_kawamura.py:22-38, tests/test_he3.py:23-69,
tests/test_he3_energy_difference.py:16-44) so the same references check both
the oracle (CPU) and the CUDA kernels.
"""

import numpy as np


def ising(spins, J):
    s = spins.astype(np.int64)
    equal = (np.sum(s == np.roll(s, -1, axis=1), axis=(1, 2))
             + np.sum(s == np.roll(s, -1, axis=2), axis=(1, 2)))
    L = s.shape[1]
    return {
        "energy": float(J) * (2 * L**2 - 2 * equal),
        "magnetization": s.sum(axis=(1, 2)).astype(np.float64),
    }


def xy(state, J):
    spins = np.exp(1j * state.astype(np.float64))
    bx = spins * np.conj(np.roll(spins, -1, axis=1))
    by = spins * np.conj(np.roll(spins, -1, axis=2))
    return {
        "energy": -float(J) * np.sum(bx.real + by.real, axis=(1, 2)),
        "mx": np.sum(spins.real, axis=(1, 2)),
        "my": np.sum(spins.imag, axis=(1, 2)),
        "twist_cos_x": np.sum(bx.real, axis=(1, 2)),
        "twist_sin_x": np.sum(bx.imag, axis=(1, 2)),
    }


def kawamura(state, J):
    state = state.astype(np.float64)
    theta, tau, d = state[..., 0], state[..., 1], state[..., 2:]
    phase = np.exp(1j * theta)
    bonds = []
    for axis in (1, 2):
        w = (1 + tau * np.roll(tau, -1, axis)) * np.sum(d * np.roll(d, -1, axis), axis=-1)
        bonds.append(w * phase * np.conj(np.roll(phase, -1, axis)))
    tensor = np.sum(d[..., :, None] * d[..., None, :] - np.eye(3) / 3, axis=(1, 2))
    return {
        "energy": -float(J) * np.sum(bonds[0].real + bonds[1].real, axis=(1, 2)),
        "chirality": tau.sum(axis=(1, 2)),
        "px": (phase**2).real.sum(axis=(1, 2)),
        "py": (phase**2).imag.sum(axis=(1, 2)),
        "spin2": np.sum(tensor**2, axis=(1, 2)) / 3,
        "twist_cos_x": bonds[0].real.sum(axis=(1, 2)),
        "twist_sin_x": bonds[0].imag.sum(axis=(1, 2)),
    }


def he3_dipole(psi):
    psi = np.asarray(psi, dtype=np.complex128)
    m = np.zeros(psi.shape[:-2] + (3, 3), dtype=np.complex128)
    m[..., :, :2] = psi
    return (np.abs(np.trace(m, axis1=-2, axis2=-1))**2
            + np.einsum("...ij,...ji->...", m, m.conj()).real
            - (2 / 3) * np.sum(np.abs(m)**2, axis=(-2, -1)))


def he3_potential(psi, coefficients, g_d=0.0):
    """Spin-matrix potential per site and the magnitude scale of its terms."""
    psi = np.asarray(psi, dtype=np.complex128)
    n = np.sum(np.abs(psi)**2, axis=(-2, -1))
    Q = np.einsum("...ma,...na->...mn", psi, psi)
    G = np.einsum("...ma,...na->...mn", psi, psi.conj())
    inv = (np.abs(np.trace(Q, axis1=-2, axis2=-1))**2, n**2, np.sum(np.abs(Q)**2, axis=(-2, -1)),
           np.sum(np.abs(G)**2, axis=(-2, -1)), np.sum((G**2).real, axis=(-2, -1)))
    terms = [-2 * n] + [float(b) * x for b, x in zip(coefficients, inv)] + [g_d * he3_dipole(psi)]
    return sum(terms), sum(np.abs(t) for t in terms)


def he3_energy(state, K, coefficients, twist=(0.0, 0.0), g_d=0.0):
    psi = np.asarray(state, dtype=np.complex128)
    pot, _ = he3_potential(psi, coefficients, g_d)
    dx = np.exp(-1j * twist[0]) * np.roll(psi, -1, axis=1) - psi
    dy = np.exp(-1j * twist[1]) * np.roll(psi, -1, axis=2) - psi
    g1 = np.sum(np.abs(dx)**2 + np.abs(dy)**2, axis=(-2, -1))
    g2 = np.sum(np.abs(dx[..., 0] + dy[..., 1])**2, axis=-1)
    g3 = np.sum(np.abs(dx[..., 0])**2 + np.abs(dy[..., 1])**2
                + 2 * (dx[..., 1].conj() * dy[..., 0]).real, axis=-1)
    return np.sum(pot + K * (g1 + g2 + g3), axis=(1, 2))


def he3_energy_parts(state, coefficients):
    psi = np.asarray(state, dtype=np.complex128)
    pot, _ = he3_potential(psi, coefficients)
    dx = np.roll(psi, -1, axis=1) - psi
    dy = np.roll(psi, -1, axis=2) - psi
    g1 = np.sum(np.abs(dx)**2 + np.abs(dy)**2, axis=(-2, -1))
    g2 = np.sum(np.abs(dx[..., 0] + dy[..., 1])**2, axis=-1)
    g3 = np.sum(np.abs(dx[..., 0])**2 + np.abs(dy[..., 1])**2
                + 2 * (dx[..., 1].conj() * dy[..., 0]).real, axis=-1)
    return pot.sum(axis=(1, 2)), (g1 + g2 + g3).sum(axis=(1, 2))


def he3(state, K, coefficients, g_d=0.0):
    psi = np.asarray(state, dtype=np.complex128)
    phase = np.sum(psi[..., 0]**2 - psi[..., 1]**2, axis=-1)
    return {
        "energy": he3_energy(psi, K, coefficients, g_d=g_d),
        "density": np.sum(np.abs(psi)**2, axis=(1, 2, 3, 4)),
        "chirality": 2 * np.sum((psi[..., 0].conj() * psi[..., 1]).imag, axis=(1, 2, 3)),
        "phase_real": phase.real.sum(axis=(1, 2)),
        "phase_imag": phase.imag.sum(axis=(1, 2)),
        "spin_alignment": 0.5 * (3 * np.sum(np.abs(psi[..., 2, :])**2, axis=(1, 2, 3))
                                 / np.sum(np.abs(psi)**2, axis=(1, 2, 3, 4)) - 1),
    }


def ising_beta_limit_colour(expected, color, hot):
    """In-place CPU update of one colour at beta = 1e8 (cold) or 0 (hot):
    tests/test_simulation.py:118-129."""
    R, L = expected.shape[:2]
    for r in range(R):
        for i in range(color // 2, L, 2):
            for j in range(color % 2, L, 2):
                nb = (int(expected[r, (i - 1) % L, j]) + int(expected[r, (i + 1) % L, j])
                      + int(expected[r, i, (j - 1) % L]) + int(expected[r, i, (j + 1) % L]))
                if hot[r] or expected[r, i, j] * nb <= 0:
                    expected[r, i, j] *= -1


def random_kawamura(rng, R, L):
    state = np.empty((R, L, L, 5), dtype=np.float32)
    state[..., 0] = rng.uniform(-np.pi, np.pi, (R, L, L))
    state[..., 1] = rng.choice([-1, 1], (R, L, L))
    d = rng.normal(size=(R, L, L, 3))
    state[..., 2:] = d / np.linalg.norm(d, axis=-1, keepdims=True)
    return state


def random_he3(rng, shape, scale=0.3):
    return (scale * (rng.normal(size=shape) + 1j * rng.normal(size=shape))).astype(np.complex64)
