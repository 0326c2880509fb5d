"""``numba.cuda.random`` on the CPU: per-thread xoroshiro128+ streams.

Restated from the published generator (Blackman & Vigna, xoroshiro128+ with
rotation/shift constants 55, 14, 36 and its 2^64 jump polynomial) and the
behaviour Numba documents for ``create_xoroshiro128p_states``: stream 0 is
seeded from one SplitMix64 output, stream k is stream k-1 advanced by one
jump, ``subsequence_start`` jumps first.  A float64 uniform is the top 53
bits times 2^-53; the float32 uniform is that float64 rounded to float32.
"""

import numpy as np

from . import to_device

xoroshiro128p_dtype = np.dtype([("s0", np.uint64), ("s1", np.uint64)], align=True)
xoroshiro128p_type = xoroshiro128p_dtype

_M64 = (1 << 64) - 1
_JUMP = (0xBEAC0467EBA5FACB, 0xD86B048B86AA9922)


def _rotl(x, k):
    return ((x << k) | (x >> (64 - k))) & _M64


def _step(s0, s1):
    """One generator step: (output, new s0, new s1)."""
    out = (s0 + s1) & _M64
    s1 ^= s0
    return out, _rotl(s0, 55) ^ s1 ^ ((s1 << 14) & _M64), _rotl(s1, 36)


def _splitmix64(seed):
    z = (seed + 0x9E3779B97F4A7C15) & _M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
    return z ^ (z >> 31)


def _jumped(s0, s1):
    a = b = 0
    for word in _JUMP:
        for bit in range(64):
            if (word >> bit) & 1:
                a ^= s0
                b ^= s1
            _, s0, s1 = _step(s0, s1)
    return a, b


def init_xoroshiro128p_states(states, seed, subsequence_start=0, stream=0):
    host = states.view(np.ndarray) if hasattr(states, "view") else states
    z = _splitmix64(int(seed) & _M64)
    s0, s1 = z, z
    for _ in range(int(subsequence_start)):
        s0, s1 = _jumped(s0, s1)
    for i in range(host.shape[0]):
        if i:
            s0, s1 = _jumped(s0, s1)
        host[i] = (s0, s1)


def create_xoroshiro128p_states(n, seed, subsequence_start=0, stream=0):
    states = to_device(np.zeros(int(n), dtype=xoroshiro128p_dtype))
    init_xoroshiro128p_states(states, seed, subsequence_start, stream)
    return states


def xoroshiro128p_next(states, index):
    rec = states[int(index)]
    out, s0, s1 = _step(int(rec["s0"]), int(rec["s1"]))
    states[int(index)] = (s0, s1)
    return np.uint64(out)


def xoroshiro128p_jump(states, index):
    rec = states[int(index)]
    states[int(index)] = _jumped(int(rec["s0"]), int(rec["s1"]))


def _unit_f64(x):
    return np.float64((int(x) >> 11) * 2.0 ** -53)


def xoroshiro128p_uniform_float64(states, index):
    return _unit_f64(xoroshiro128p_next(states, index))


def xoroshiro128p_uniform_float32(states, index):
    return np.float32(_unit_f64(xoroshiro128p_next(states, index)))
