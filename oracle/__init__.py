"""CPU oracle for the lattice Monte Carlo hot path — test infrastructure only.

A C restatement (``mc_oracle.c``) of the reference's Numba-CUDA kernels, loaded
through ctypes.  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline leg import this package; the product path (``mcgb``) never does.

Each wrapper takes and returns NumPy arrays in the reference's layouts:
state ``(R, L, L, ...)``, RNG states ``(n, 2)`` uint64 (``s0, s1``), betas
``(R,)`` float32, measurement outputs ``(C, R)`` float64.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libmc_oracle.so"

_lib = None


def build(force: bool = False) -> Path:
    """Compile the oracle with gcc (a second or two)."""
    src = HERE / "mc_oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
               "-fopenmp", "-shared", "-o", str(LIB_PATH), str(src), "-lm"]
        subprocess.run(cmd, check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIB_PATH))
        _declare(_lib)
    return _lib


_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_F = ctypes.c_float


def _declare(L):
    sig = {
        "orc_rng_init": (None, [_P, _I64, _U64, _U64]),
        "orc_rng_next": (_U64, [_P]),
        "orc_rng_jump": (None, [_P]),
        "orc_rng_uniform_f32": (_F, [_P]),
        "orc_rng_uniform_f64": (ctypes.c_double, [_P]),
        "orc_splitmix64_first": (_U64, [_U64]),
        "orc_ising_update_color": (None, [_P, _P, _P, _I, _I, _I, _F]),
        "orc_ising_sweeps": (None, [_P, _P, _P, _I, _I, _F, _I, _I]),
        "orc_ising_sweeps_tab": (None, [_P, _P, _P, _P, _I, _I, _F, _I, _I]),
        "orc_ising_energy": (None, [_P, _I, _I, _F, _P]),
        "orc_ising_measure": (None, [_P, _I, _I, _F, _P, _P, _P]),
        "orc_xy_update_color": (None, [_P, _P, _P, _I, _I, _I, _F, _F]),
        "orc_xy_update_color_gauss": (None, [_P, _P, _P, _P, _I, _I, _I, _F]),
        "orc_xy_sweeps": (None, [_P, _P, _P, _P, _I, _I, _F, _F, _I, _I]),
        "orc_xy_energy": (None, [_P, _I, _I, _F, _P]),
        "orc_xy_measure": (None, [_P, _I, _I, _F, _P, _P, _P]),
        "orc_kawamura_local_energy": (_F, [_P, _I, _I, _I, _I, _F, _F, _F, _F, _F, _F]),
        "orc_kawamura_update_color": (None, [_P, _P, _P, _I, _I, _I, _F, _F]),
        "orc_kawamura_sweeps": (None, [_P, _P, _P, _I, _I, _F, _F, _I, _I]),
        "orc_kawamura_update_color_gauss": (None, [_P, _P, _P, _P, _I, _I, _I, _F]),
        "orc_kawamura_sweeps_gauss": (None, [_P, _P, _P, _P, _I, _I, _F, _I, _I]),
        "orc_kawamura_energy": (None, [_P, _I, _I, _F, _P]),
        "orc_kawamura_measure": (None, [_P, _I, _I, _F, _P, _P, _P]),
        "orc_he3_potential": (_F, [_P, _P, _F]),
        "orc_he3_gradient_difference": (_F, [_P, _I, _I, _I, _I, _P]),
        "orc_he3_update_color": (None, [_P, _P, _P, _I, _I, _I, _P, _F, _F, _F]),
        "orc_he3_gaussian_update_color": (None, [_P, _P, _P, _I, _I, _I, _P, _F, _F, _F, _F, _P]),
        "orc_he3_sweeps": (None, [_P, _P, _P, _I, _I, _P, _F, _F, _F, _I, _F, _F, _P, _I, _I]),
        "orc_he3_energy": (None, [_P, _I, _I, _P, _F, _F, _P]),
        "orc_he3_measure": (None, [_P, _I, _I, _P, _F, _F, _P, _P, _P]),
        "orc_pt_exchange": (None, [_P, _P, _P, _P, _P, _P, _P, _I, _I, _I64]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _check(a, dtype, name):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        raise TypeError(f"{name} must be a C-contiguous {np.dtype(dtype)} ndarray")
    return a


# ---------------------------------------------------------------- RNG


def rng_states(n: int, seed: int, subsequence_start: int = 0) -> np.ndarray:
    """Sequential-jump initialisation, as numba.cuda.random does on the host."""
    out = np.zeros((n, 2), dtype=np.uint64)
    lib().orc_rng_init(_ptr(out), n, seed & (2**64 - 1), subsequence_start)
    return out


def splitmix64_first(seed: int) -> int:
    return int(lib().orc_splitmix64_first(seed & (2**64 - 1)))


def rng_next(state: np.ndarray) -> int:
    _check(state, np.uint64, "state")
    return int(lib().orc_rng_next(_ptr(state)))


def rng_jump(state: np.ndarray) -> None:
    _check(state, np.uint64, "state")
    lib().orc_rng_jump(_ptr(state))


def uniform_f32(state: np.ndarray) -> float:
    return float(lib().orc_rng_uniform_f32(_ptr(_check(state, np.uint64, "state"))))


def uniform_f64(state: np.ndarray) -> float:
    return float(lib().orc_rng_uniform_f64(_ptr(_check(state, np.uint64, "state"))))


# ---------------------------------------------------------------- models


def _idx(t):
    return None if t is None else np.ascontiguousarray(t, dtype=np.int32)


def _cache(c):
    return None if c is None else np.ascontiguousarray(c, dtype=np.float64)


def ising_update_color(spins, rng, betas, color, J):
    R, L = spins.shape[0], spins.shape[1]
    lib().orc_ising_update_color(_ptr(_check(spins, np.int8, "spins")), _ptr(_check(rng, np.uint64, "rng")),
                                 _ptr(_check(betas, np.float32, "betas")), R, L, color, J)


def ising_sweeps(spins, rng, betas, J, n_sweeps, n_threads=1):
    R, L = spins.shape[0], spins.shape[1]
    lib().orc_ising_sweeps(_ptr(_check(spins, np.int8, "spins")), _ptr(_check(rng, np.uint64, "rng")),
                           _ptr(_check(betas, np.float32, "betas")), R, L, J, n_sweeps, n_threads)


def ising_exponent_arguments(betas, J):
    """float32 arguments -beta * (float32(k) * J), k = -8, -4, 0, 4, 8, shape (R, 5)."""
    k = np.array([-8, -4, 0, 4, 8], dtype=np.float32)
    return (-np.asarray(betas, np.float32)[:, None] * (k[None, :] * np.float32(J))).astype(np.float32)


def ising_sweeps_tab(spins, rng, betas, table, J, n_sweeps, n_threads=1):
    """Sweeps whose acceptance exponentials come from ``table`` (R, 5) float32."""
    R, L = spins.shape[0], spins.shape[1]
    tab = np.ascontiguousarray(table, dtype=np.float32)
    if tab.shape != (R, 5):
        raise ValueError("table must have shape (R, 5)")
    lib().orc_ising_sweeps_tab(_ptr(_check(spins, np.int8, "spins")), _ptr(_check(rng, np.uint64, "rng")),
                               _ptr(_check(betas, np.float32, "betas")), _ptr(tab), R, L, J, n_sweeps,
                               n_threads)


def ising_energy(spins, J):
    R, L = spins.shape[0], spins.shape[1]
    out = np.zeros(R)
    lib().orc_ising_energy(_ptr(_check(spins, np.int8, "spins")), R, L, J, _ptr(out))
    return out


def ising_measure(spins, J, temperature_indices=None, cached=None):
    R, L = spins.shape[0], spins.shape[1]
    out = np.zeros((2, R))
    t, c = _idx(temperature_indices), _cache(cached)
    lib().orc_ising_measure(_ptr(_check(spins, np.int8, "spins")), R, L, J, _ptr(t), _ptr(c), _ptr(out))
    return out


def xy_update_color(theta, rng, betas, color, J, delta):
    R, L = theta.shape[0], theta.shape[1]
    lib().orc_xy_update_color(_ptr(_check(theta, np.float32, "theta")), _ptr(_check(rng, np.uint64, "rng")),
                              _ptr(_check(betas, np.float32, "betas")), R, L, color, J, delta)


def xy_update_color_gauss(theta, rng, betas, sigmas, color, J):
    R, L = theta.shape[0], theta.shape[1]
    lib().orc_xy_update_color_gauss(_ptr(_check(theta, np.float32, "theta")),
                                    _ptr(_check(rng, np.uint64, "rng")),
                                    _ptr(_check(betas, np.float32, "betas")),
                                    _ptr(_check(sigmas, np.float32, "sigmas")), R, L, color, J)


def xy_sweeps(theta, rng, betas, J, delta, n_sweeps, sigmas=None, n_threads=1):
    R, L = theta.shape[0], theta.shape[1]
    s = None if sigmas is None else _check(sigmas, np.float32, "sigmas")
    lib().orc_xy_sweeps(_ptr(_check(theta, np.float32, "theta")), _ptr(_check(rng, np.uint64, "rng")),
                        _ptr(_check(betas, np.float32, "betas")), _ptr(s), R, L, J, delta,
                        n_sweeps, n_threads)


def xy_energy(theta, J):
    R, L = theta.shape[0], theta.shape[1]
    out = np.zeros(R)
    lib().orc_xy_energy(_ptr(_check(theta, np.float32, "theta")), R, L, J, _ptr(out))
    return out


def xy_measure(theta, J, temperature_indices=None, cached=None):
    R, L = theta.shape[0], theta.shape[1]
    out = np.zeros((5, R))
    t, c = _idx(temperature_indices), _cache(cached)
    lib().orc_xy_measure(_ptr(_check(theta, np.float32, "theta")), R, L, J, _ptr(t), _ptr(c), _ptr(out))
    return out


def kawamura_local_energy(state, r, i, j, site, J):
    L = state.shape[1]
    return float(lib().orc_kawamura_local_energy(_ptr(_check(state, np.float32, "state")), L, r, i, j,
                                                 *[float(v) for v in site], J))


def kawamura_update_color(state, rng, betas, color, J, delta):
    R, L = state.shape[0], state.shape[1]
    lib().orc_kawamura_update_color(_ptr(_check(state, np.float32, "state")), _ptr(_check(rng, np.uint64, "rng")),
                                    _ptr(_check(betas, np.float32, "betas")), R, L, color, J, delta)


def kawamura_sweeps(state, rng, betas, J, delta, n_sweeps, n_threads=1):
    R, L = state.shape[0], state.shape[1]
    lib().orc_kawamura_sweeps(_ptr(_check(state, np.float32, "state")), _ptr(_check(rng, np.uint64, "rng")),
                              _ptr(_check(betas, np.float32, "betas")), R, L, J, delta, n_sweeps, n_threads)


def kawamura_update_color_gauss(state, rng, betas, sigmas, color, J):
    R, L = state.shape[0], state.shape[1]
    lib().orc_kawamura_update_color_gauss(_ptr(_check(state, np.float32, "state")), _ptr(_check(rng, np.uint64, "rng")),
                                          _ptr(_check(betas, np.float32, "betas")),
                                          _ptr(_check(sigmas, np.float32, "sigmas")), R, L, color, J)


def kawamura_sweeps_gauss(state, rng, betas, sigmas, J, n_sweeps, n_threads=1):
    R, L = state.shape[0], state.shape[1]
    lib().orc_kawamura_sweeps_gauss(_ptr(_check(state, np.float32, "state")), _ptr(_check(rng, np.uint64, "rng")),
                                    _ptr(_check(betas, np.float32, "betas")),
                                    _ptr(_check(sigmas, np.float32, "sigmas")), R, L, J, n_sweeps, n_threads)


def kawamura_energy(state, J):
    R, L = state.shape[0], state.shape[1]
    out = np.zeros(R)
    lib().orc_kawamura_energy(_ptr(_check(state, np.float32, "state")), R, L, J, _ptr(out))
    return out


def kawamura_measure(state, J, temperature_indices=None, cached=None):
    R, L = state.shape[0], state.shape[1]
    out = np.zeros((7, R))
    t, c = _idx(temperature_indices), _cache(cached)
    lib().orc_kawamura_measure(_ptr(_check(state, np.float32, "state")), R, L, J, _ptr(t), _ptr(c), _ptr(out))
    return out


def _c64(state):
    if state.dtype != np.complex64 or not state.flags.c_contiguous:
        raise TypeError("He3 state must be a C-contiguous complex64 ndarray")
    return state


def _coeff(coefficients):
    return np.ascontiguousarray(np.asarray(coefficients, dtype=np.float32))


def he3_potential(psi, coefficients, g_d=0.0):
    psi = np.ascontiguousarray(psi, dtype=np.complex64)
    return float(lib().orc_he3_potential(_ptr(psi), _ptr(_coeff(coefficients)), g_d))


def he3_gradient_difference(state, r, i, j, proposed):
    p = np.ascontiguousarray(proposed, dtype=np.complex64)
    return float(lib().orc_he3_gradient_difference(_ptr(_c64(state)), state.shape[1], r, i, j, _ptr(p)))


def he3_update_color(state, rng, betas, color, coefficients, K, delta, g_d):
    R, L = state.shape[0], state.shape[1]
    lib().orc_he3_update_color(_ptr(_c64(state)), _ptr(_check(rng, np.uint64, "rng")),
                               _ptr(_check(betas, np.float32, "betas")), R, L, color,
                               _ptr(_coeff(coefficients)), K, delta, g_d)


def he3_gaussian_update_color(state, rng, betas, color, coefficients, K, rho, mass, g_d, counts):
    R, L = state.shape[0], state.shape[1]
    lib().orc_he3_gaussian_update_color(_ptr(_c64(state)), _ptr(_check(rng, np.uint64, "rng")),
                                        _ptr(_check(betas, np.float32, "betas")), R, L, color,
                                        _ptr(_coeff(coefficients)), K, rho, mass, g_d,
                                        _ptr(_check(counts, np.int64, "counts")))


def he3_sweeps(state, rng, betas, coefficients, K, delta, g_d, n_sweeps, gaussian=False,
               rho=-0.9, mass=0.0, counts=None, n_threads=1):
    R, L = state.shape[0], state.shape[1]
    if gaussian and counts is None:
        counts = np.zeros((3, R, L, L), dtype=np.int64)
    lib().orc_he3_sweeps(_ptr(_c64(state)), _ptr(_check(rng, np.uint64, "rng")),
                         _ptr(_check(betas, np.float32, "betas")), R, L, _ptr(_coeff(coefficients)),
                         K, delta, g_d, int(gaussian), rho, mass, _ptr(counts), n_sweeps, n_threads)
    return counts


def he3_energy(state, coefficients, K, g_d=0.0):
    R, L = state.shape[0], state.shape[1]
    out = np.zeros(R)
    lib().orc_he3_energy(_ptr(_c64(state)), R, L, _ptr(_coeff(coefficients)), K, g_d, _ptr(out))
    return out


def he3_measure(state, coefficients, K, g_d=0.0, temperature_indices=None, cached=None):
    R, L = state.shape[0], state.shape[1]
    out = np.zeros((10, R))
    t, c = _idx(temperature_indices), _cache(cached)
    lib().orc_he3_measure(_ptr(_c64(state)), R, L, _ptr(_coeff(coefficients)), K, g_d,
                          _ptr(t), _ptr(c), _ptr(out))
    return out


# ---------------------------------------------------------------- PT


def pt_exchange(energies, betas, w2t, t2w, rng, swap_counts, trips, parity, sweep):
    R = len(energies)
    lib().orc_pt_exchange(_ptr(_check(energies, np.float64, "energies")), _ptr(_check(betas, np.float32, "betas")),
                          _ptr(_check(w2t, np.int32, "w2t")), _ptr(_check(t2w, np.int32, "t2w")),
                          _ptr(_check(rng, np.uint64, "rng")), _ptr(_check(swap_counts, np.int64, "swap_counts")),
                          _ptr(_check(trips, np.int64, "trips")), R, parity, sweep)


def pt_initial_trips(R):
    """Round-trip bookkeeping as core/parallel_tempering.py:182-187 seeds it."""
    trips = np.zeros((5, R), dtype=np.int64)
    trips[0] = -1
    trips[2] = -1
    trips[0, 0] = 0
    trips[0, -1] = R - 1
    trips[2, [0, -1]] = 0
    return trips


n_cpu = os.cpu_count() or 1
