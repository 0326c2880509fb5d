"""Shared helpers for the fixtures written by the reference's own kernels
(tests/golden/reference_kernels.npz, made by
tests/golden/make_reference_kernel_golden.py under the numba stand-in).

Tolerances, used by the oracle test (CPU) and the CUDA test (GPU):

* Ising lattices, every RNG stream, exchange maps, swap and round-trip
  counters, walker histories and sample sweeps: exact;
* continuous states: within STATE_TOL = 1e-5 per component, except that an
  accept/reject decision may differ at a site whose uniform lies within
  rounding of the acceptance probability (the stand-in's transcendentals are
  the correctly rounded float32 values, CUDA's within 2 ulp): at most
  MAX_FLIP_FRACTION of the sites;
* measurement channels of the same final state: MEASURE_RTOL = 1e-9
  relative (float64 sums in another order), 1e-6 for He3, whose per-site
  terms are float32; samples along a continuous trajectory: SAMPLE_RTOL.
"""

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
STATE_TOL = 1e-5
MAX_FLIP_FRACTION = 1e-3
MEASURE_RTOL = {"ising": 0.0, "xy": 1e-9, "kawamura": 1e-9, "he3": 1e-6}
SAMPLE_RTOL = {"ising": 0.0, "xy": 1e-5, "kawamura": 1e-5, "he3": 1e-5}

RUNTIME_CASES = ("ising_rt", "xy_rt", "kawamura_rt", "he3_rt", "he3p_rt", "he3g_rt")
PT_CASES = ("ising_pt", "xy_pt", "kawamura_pt", "he3_pt")


def load():
    return dict(np.load(GOLDEN / "reference_kernels.npz"))


def expf_table():
    cap = json.loads((GOLDEN / "ising_cuda_expf.json").read_text())
    return {int(a, 16): int(v, 16) for args, vals in zip(cap["arguments_f32_bits"], cap["expf_f32_bits"])
            for a, v in zip(args, vals)}


def case(fx, name):
    """The arrays of one case, keys relative to it; scalars unwrapped."""
    pre = name + "/"
    out = {}
    for k, v in fx.items():
        if k.startswith(pre):
            out[k[len(pre):]] = v.item() if v.ndim == 0 and v.dtype.kind in "iuf" else v
    out["kind"] = str(fx[pre + "kind"])
    return out


def channel(c, group):
    pre = group + "/"
    return {k[len(pre):]: v for k, v in c.items() if k.startswith(pre)}


def params(c):
    return channel(c, "params")


def family(kind):
    return "he3" if kind.startswith("he3") else kind


def assert_states_close(got, ref, kind):
    if kind == "ising":
        np.testing.assert_array_equal(got, ref)
        return
    diff = np.abs(np.asarray(got).astype(np.complex128) - np.asarray(ref).astype(np.complex128))
    R, L = diff.shape[0], diff.shape[1]
    site = diff.reshape(R, L, L, -1).max(axis=-1)
    bad = site > STATE_TOL
    assert bad.mean() <= MAX_FLIP_FRACTION, f"{bad.sum()} of {bad.size} sites differ (max {site.max():.3g})"


def assert_rng_equal(got, ref):
    got = np.asarray(got)
    if got.dtype.names:
        got = np.stack([got["s0"], got["s1"]], axis=-1)
    ref = np.stack([ref["s0"], ref["s1"]], axis=-1) if ref.dtype.names else ref
    np.testing.assert_array_equal(got.astype(np.uint64), ref.astype(np.uint64))


def assert_channels_close(got, ref, rtol, what):
    assert set(got) == set(ref), (sorted(got), sorted(ref))
    for ch in ref:
        g, r = np.asarray(got[ch], np.float64), np.asarray(ref[ch], np.float64)
        if rtol == 0.0:
            np.testing.assert_array_equal(g, r, err_msg=f"{what} {ch}")
        else:
            scale = max(1.0, float(np.abs(r).max()))
            np.testing.assert_allclose(g, r, rtol=rtol, atol=rtol * scale, err_msg=f"{what} {ch}")


PT_EXACT = ("attempts", "accepted", "walker_to_temperature", "temperature_to_walker", "walker_round_trips",
            "walker_round_trip_total_sweeps", "exchange_rounds", "sweeps", "next_parity", "exchange_seed")
