"""Write the golden fixtures of this directory.

    python tests/golden/make_golden.py

* ``rng_streams.json`` -- xoroshiro128+ streams as ``numba.cuda.random``
  seeds them (SplitMix64 of the seed fills both words of stream 0; stream k
  is stream k-1 advanced by the 2^64 jump), from the pure-Python restatement
  below, written independently of the C oracle: raw 64-bit outputs and the
  float64/float32 uniforms (top 53 bits x 2^-53, the float32 one rounded
  from the float64), for several seeds and stream indices.
* ``sweeps.npz`` -- small seeded runs of every update rule (and of the XY and
  Kawamura Gaussian proposals) through the C
  oracle (the reference kernels restated): inputs, final states and RNG
  streams after a few four-colour sweeps, and the measurement channels of
  the final states.
* ``pt.npz`` -- a sequence of replica-exchange rounds through the oracle's
  restatement of the exchange kernel: maps, betas, counters and round-trip
  bookkeeping after every round.

The Ising acceptance exponentials are an input of the sweep: the reference
evaluates CUDA's float32 ``expf``, which is not correctly rounded at every
argument.  ``ising_cuda_expf.json`` (written on a GPU by
``capture_cuda_expf.py``) holds CUDA's values for the fixture's arguments;
the fixture stores that table with the sweep it drove.
"""

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

import oracle  # noqa: E402

M64 = (1 << 64) - 1


# ----------------------------------------------------------- pure-Python RNG

def _rotl(x, k):
    return ((x << k) | (x >> (64 - k))) & M64


def splitmix64(seed):
    z = (seed + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def next_raw(s):
    """Advance [s0, s1] in place, return the output s0 + s1."""
    s0, s1 = s
    out = (s0 + s1) & M64
    s1 ^= s0
    s[0] = _rotl(s0, 55) ^ s1 ^ ((s1 << 14) & M64)
    s[1] = _rotl(s1, 36)
    return out


JUMP = (0xBEAC0467EBA5FACB, 0xD86B048B86AA9922)


def jump(s):
    a = b = 0
    for word in JUMP:
        for bit in range(64):
            if (word >> bit) & 1:
                a ^= s[0]
                b ^= s[1]
            next_raw(s)
    s[0], s[1] = a, b


def stream(seed, k):
    z = splitmix64(seed)
    s = [z, z]
    for _ in range(k):
        jump(s)
    return s


def rng_fixture():
    seeds = [0, 1, 42, 106, 1234567, 2 ** 40 + 5]
    indices = [0, 1, 2, 7, 100, 1023]
    cases = []
    for seed in seeds:
        s = stream(seed, 0)
        done = 0
        for k in indices:
            while done < k:
                jump(s)
                done += 1
            st = list(s)
            raw = [next_raw(st) for _ in range(4)]
            st = list(s)
            f64 = [float(np.float64(next_raw(st) >> 11) * np.float64(2.0 ** -53)) for _ in range(4)]
            f32 = [int(np.float32(x).view(np.uint32)) for x in f64]
            cases.append({"seed": seed, "stream": k, "state": [f"{v:016x}" for v in s],
                          "raw": [f"{v:016x}" for v in raw], "uniform_f64": [x.hex() for x in f64],
                          "uniform_f32_bits": [f"{v:08x}" for v in f32]})
    return {"generator": "xoroshiro128+ (55, 14, 36), SplitMix64 seeding, 2^64 jump per stream",
            "cases": cases}


# ----------------------------------------------------------- sweeps

def cuda_ising_table(temperatures):
    """CUDA's expf of the five acceptance arguments per temperature, (R, 5)."""
    cap = json.loads((HERE / "ising_cuda_expf.json").read_text())
    if list(cap["temperatures"]) != list(temperatures):
        raise ValueError("ising_cuda_expf.json was captured for other temperatures")
    args = oracle.ising_exponent_arguments((1 / np.asarray(temperatures)).astype(np.float32), 1.0)
    captured = np.array([[int(v, 16) for v in row] for row in cap["arguments_f32_bits"]], np.uint32)
    if not np.array_equal(args.view(np.uint32), captured):
        raise ValueError("captured arguments differ from the oracle's")
    return np.array([[int(v, 16) for v in row] for row in cap["expf_f32_bits"]], np.uint32).view(np.float32)


def sweep_fixture():
    out = {}
    r = np.random.default_rng(20260101)

    # Ising: L=16, three temperatures of the L=64 study, 10 sweeps.
    L, T, seed = 16, [1.5, 2.269, 3.0], 58
    betas = (1 / np.asarray(T)).astype(np.float32)
    spins = r.choice(np.array([-1, 1], np.int8), (3, L, L))
    table = cuda_ising_table(T)
    state, rng = spins.copy(), oracle.rng_states(3 * L * L, seed)
    oracle.ising_sweeps_tab(state, rng, betas, table, np.float32(1), 10)
    out.update({"ising_seed": seed, "ising_betas": betas, "ising_in": spins, "ising_table": table,
                "ising_sweeps": 10, "ising_out": state, "ising_rng_out": rng,
                "ising_measure": oracle.ising_measure(state, np.float32(1))})

    # XY: uniform delta = 1.5 and Gaussian proposals, 5 sweeps.
    L, T, seed = 16, np.array([0.8, 1.1]), 60
    betas = (1 / T).astype(np.float32)
    theta = r.uniform(-np.pi, np.pi, (2, L, L)).astype(np.float32)
    sig = np.array([0.9, 1.3], np.float32)
    for name, sigmas in (("xy", None), ("xyg", sig)):
        state, rng = theta.copy(), oracle.rng_states(2 * L * L, seed)
        oracle.xy_sweeps(state, rng, betas, np.float32(1), np.float32(1.5), 5, sigmas=sigmas)
        out.update({f"{name}_seed": seed, f"{name}_betas": betas, f"{name}_in": theta, f"{name}_sweeps": 5,
                    f"{name}_out": state, f"{name}_rng_out": rng,
                    f"{name}_measure": oracle.xy_measure(state, np.float32(1))})
    out["xyg_sigmas"] = sig

    # Kawamura: L=8, theta uniform, tau = +-1, d a normalised Gaussian vector; 3 sweeps.
    L, T, seed = 8, np.array([0.70, 0.75]), 52
    betas = (1 / T).astype(np.float32)
    st = np.zeros((2, L, L, 5), np.float32)
    st[..., 0] = r.uniform(-np.pi, np.pi, (2, L, L))
    st[..., 1] = r.choice([-1.0, 1.0], (2, L, L))
    d = r.normal(size=(2, L, L, 3))
    st[..., 2:] = d / np.linalg.norm(d, axis=-1, keepdims=True)
    state, rng = st.copy(), oracle.rng_states(2 * L * L, seed)
    oracle.kawamura_sweeps(state, rng, betas, np.float32(1), np.float32(1.5), 3)
    out.update({"kaw_seed": seed, "kaw_betas": betas, "kaw_in": st, "kaw_sweeps": 3, "kaw_out": state,
                "kaw_rng_out": rng, "kaw_measure": oracle.kawamura_measure(state, np.float32(1))})
    # ... and with Gaussian proposals (this project's extension).
    sig = np.array([0.6, 0.8], np.float32)
    state, rng = st.copy(), oracle.rng_states(2 * L * L, seed)
    oracle.kawamura_sweeps_gauss(state, rng, betas, sig, np.float32(1), 3)
    out.update({"kawg_sigmas": sig, "kawg_out": state, "kawg_rng_out": rng})

    # He3 (class defaults): Cartesian and conditional-Gaussian proposals, 2 sweeps.
    L, T, seed = 8, np.array([0.35, 0.45]), 50
    betas = (1 / T).astype(np.float32)
    coeff = np.array([-0.5, 1.0, 1.0, 1.0, -1.0], np.float32)   # He3Model() GL coefficients
    a = 0.3 * np.sqrt(2)
    psi = (r.uniform(-a, a, (2, L, L, 3, 2)) + 1j * r.uniform(-a, a, (2, L, L, 3, 2))).astype(np.complex64)
    for name, gaussian in (("he3", False), ("he3g", True)):
        state, rng = psi.copy(), oracle.rng_states(2 * L * L, seed)
        counts = oracle.he3_sweeps(state, rng, betas, coeff, np.float32(1), np.float32(0.15), np.float32(0),
                                   2, gaussian=gaussian, rho=np.float32(-0.9), mass=np.float32(0))
        out.update({f"{name}_seed": seed, f"{name}_betas": betas, f"{name}_in": psi, f"{name}_sweeps": 2,
                    f"{name}_out": state, f"{name}_rng_out": rng,
                    f"{name}_measure": oracle.he3_measure(state, coeff, np.float32(1))})
        if gaussian:
            out["he3g_counts"] = counts
    out["he3_coefficients"] = coeff
    return out


# ----------------------------------------------------------- exchange

def pt_fixture():
    R, rounds, seed = 6, 120, 7
    r = np.random.default_rng(99)
    T = np.geomspace(0.7, 1.2, R)
    betas = (1 / T).astype(np.float32)
    w2t, t2w = np.arange(R, dtype=np.int32), np.arange(R, dtype=np.int32)
    rng = oracle.rng_states(R - 1, seed)
    counts = np.zeros((3, R - 1), np.int64)
    trips = oracle.pt_initial_trips(R)
    energies = -400.0 + 40.0 * r.normal(size=(rounds, R))
    hist = {k: [] for k in ("w2t", "t2w", "betas", "counts", "trips")}
    b = betas.copy()
    for k in range(rounds):
        e = np.ascontiguousarray(energies[k])
        oracle.pt_exchange(e, b, w2t, t2w, rng, counts, trips, k & 1, 10 * (k + 1))
        for name, v in (("w2t", w2t), ("t2w", t2w), ("betas", b), ("counts", counts), ("trips", trips)):
            hist[name].append(v.copy())
    return {"seed": seed, "betas_in": betas, "energies": energies,
            **{name: np.stack(v) for name, v in hist.items()}}


def main():
    (HERE / "rng_streams.json").write_text(json.dumps(rng_fixture(), indent=1) + "\n")
    np.savez_compressed(HERE / "sweeps.npz", **sweep_fixture())
    np.savez_compressed(HERE / "pt.npz", **pt_fixture())
    for f in ("rng_streams.json", "sweeps.npz", "pt.npz"):
        print(f, (HERE / f).stat().st_size, "bytes")


if __name__ == "__main__":
    main()
