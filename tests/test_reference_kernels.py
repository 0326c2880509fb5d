"""The oracle against fixtures written by the reference's own kernels.

tests/golden/reference_kernels.npz holds runs of the reference's unmodified
Runtime, ParallelTempering, Simulation, He3GaussianRuntime and model
plugins (models/*/update.py, measure.py, models/he3/gaussian_fast.py,
core/parallel_tempering.py:35-91), executed on the CPU under the numba
stand-in (tests/golden/numba_standin).  Here the oracle's C restatement,
driven by oracle/dropin.py's replay of the same host control flow, must
reproduce them: Ising bit for bit, every RNG stream and every PT counter
exactly, continuous states and measurements within the tolerances of
tests/refcases.py.  tests/test_gpu_reference_kernels.py holds the CUDA path
to the same fixtures.
"""

import numpy as np
import pytest

import oracle
import refcases as rc
from oracle import dropin


@pytest.fixture(scope="module")
def fx():
    return rc.load()


def ops_for(c):
    p = rc.params(c)
    kind = c["kind"]
    if kind == "he3" and "rho" in p:
        kind = "he3g"
    args = {"J": p.get("J"), "delta": p.get("delta"), "K": p.get("K"), "g_d": p.get("g_d"),
            "coefficients": p.get("coefficients"), "rho": p.get("rho"), "mass": p.get("proposal_mass")}
    return dropin.ModelOps(kind, {k: (v if k == "coefficients" or v is None else np.float32(v))
                                  for k, v in args.items()}, expf_table=rc.expf_table())


@pytest.mark.parametrize("name", rc.RUNTIME_CASES)
def test_oracle_runtime_matches_reference_kernels(fx, name):
    c = rc.case(fx, name)
    ops = ops_for(c)
    rt = dropin.Runtime(ops, c["in"], c["T"], int(c["seed"]))
    np.testing.assert_array_equal(rt.betas, c["betas"])
    for _ in range(int(c["sweeps"])):
        rt.sweep()
    rc.assert_rng_equal(rt.rng, c["rng_out"])
    rc.assert_states_close(rt.state, c["out"], c["kind"])
    if ops.kind == "he3g":
        np.testing.assert_array_equal(ops.counts, c["counts"])
    # The measurements of the reference's final state.
    fam = rc.family(c["kind"])
    ref_state = np.ascontiguousarray(c["out"])
    rtol = rc.MEASURE_RTOL[fam]
    e = ops.energy(ref_state)
    np.testing.assert_allclose(e, c["energy"], rtol=rtol, atol=rtol)
    rc.assert_channels_close(ops.measure(ref_state), rc.channel(c, "measure"), rtol, name)
    rc.assert_channels_close(ops.measure(ref_state, c["measure_order"]), rc.channel(c, "measure_t"), rtol, name)


@pytest.mark.parametrize("name", rc.PT_CASES)
def test_oracle_pt_simulation_matches_reference(fx, name):
    c = rc.case(fx, name)
    ops = ops_for(c)
    rt = dropin.Runtime(ops, c["in"], c["T"], int(c["seed"]))
    pt = dropin.ParallelTempering(rt, exchange_interval=int(c["interval"]),
                                  tracked_walkers=list(c["tracked"]), history_stride=int(c["history_stride"]))
    samples, sweeps = dropin.simulate(pt, int(c["thermalization"]), int(c["measurement"]),
                                      int(c["sample_interval"]))
    np.testing.assert_array_equal(sweeps, c["sample_sweeps"])
    rc.assert_rng_equal(rt.rng, c["rng_out"])
    rc.assert_rng_equal(pt.rng, c["exchange_rng_out"])
    rc.assert_states_close(rt.state, c["out"], c["kind"])
    np.testing.assert_array_equal(rt.betas, c["betas_out"])
    ref_pt = rc.channel(c, "pt")
    got_pt = {"attempts": pt.swap_counts[0], "accepted": pt.swap_counts[1], "walker_to_temperature": pt.w2t,
              "temperature_to_walker": pt.t2w, "walker_round_trips": pt.trips[3],
              "walker_round_trip_total_sweeps": pt.trips[4], "exchange_rounds": pt.exchange_rounds,
              "sweeps": pt.sweeps, "next_parity": pt.parity, "exchange_seed": pt.exchange_seed}
    for k in rc.PT_EXACT:
        np.testing.assert_array_equal(np.asarray(got_pt[k]), np.asarray(ref_pt[k]), err_msg=k)
    hist = pt.walker_history()
    for k in ("walker_ids", "sweeps", "exchange_rounds", "temperature_indices"):
        np.testing.assert_array_equal(hist[k], ref_pt[f"history/{k}"], err_msg=k)
    rc.assert_channels_close(samples, rc.channel(c, "samples"), rc.SAMPLE_RTOL[rc.family(c["kind"])], name)
    np.testing.assert_allclose(pt.energies, c["energies"], rtol=rc.SAMPLE_RTOL[rc.family(c["kind"])])


def test_fixture_covers_every_model_and_the_pt_path(fx):
    kinds = {str(fx[f"{n}/kind"]) for n in rc.RUNTIME_CASES + rc.PT_CASES}
    assert kinds == {"ising", "xy", "kawamura", "he3"}
    # Exchanges were accepted and rejected in every PT case, so both branches are pinned.
    for n in rc.PT_CASES:
        acc, att = fx[f"{n}/pt/accepted"], fx[f"{n}/pt/attempts"]
        assert acc.sum() > 0 and (att - acc).sum() > 0, n


def test_dropin_he3_pressure_coefficients_match_reference(fx):
    """The drop-in He3Model's strong-coupling correction gives the reference
    model's float32 coefficients at the fixture's pressure."""
    from mcgb.models.he3.model import He3Model
    p = rc.params(rc.case(fx, "he3p_rt"))
    m = He3Model(pressure=float(p["pressure"]), reduced_temperature=float(p["reduced_temperature"]),
                 g_d=float(p["g_d"]))
    np.testing.assert_array_equal(np.asarray(m.betas, np.float32), p["coefficients"])
    np.testing.assert_array_equal(np.float32(m.g_d), p["g_d"])
