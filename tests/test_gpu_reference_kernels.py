"""The CUDA path against fixtures written by the reference's own kernels.

tests/golden/reference_kernels.npz holds runs of the reference's unmodified
classes and kernels (executed under the numba stand-in, see
tests/golden/make_reference_kernel_golden.py).  Each test here repeats the
same driver script with this project's drop-in classes -- Runtime,
ParallelTempering, Simulation, He3GaussianRuntime and the model plugins, all
launching the CUDA library -- and the batched engine for the Ising ladder.
Tolerances are tests/refcases.py's: Ising, RNG streams and every PT counter
exact; continuous states 1e-5; measurements 1e-9 relative (He3 1e-6).
"""

import numpy as np
import pytest

import refcases as rc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fx():
    return rc.load()


def make_model(c):
    p = rc.params(c)
    kind = c["kind"]
    if kind == "ising":
        from mcgb.models.ising.model import IsingModel
        return IsingModel(J=float(p["J"]))
    if kind == "xy":
        from mcgb.models.xy.model import XYModel
        return XYModel(J=float(p["J"]), delta=float(p["delta"]))
    if kind == "kawamura":
        from mcgb.models.kawamura.model import KawamuraModel
        return KawamuraModel(J=float(p["J"]), delta=float(p["delta"]))
    from mcgb.models.he3.model import He3Model
    kw = {}
    if "pressure" in p:
        kw = {"pressure": float(p["pressure"]), "reduced_temperature": float(p["reduced_temperature"])}
    m = He3Model(K=float(p["K"]), delta=float(p["delta"]), g_d=float(p["g_d"]), **kw)
    # The float32 coefficients (pressure-corrected where the case set a
    # pressure) must be the reference model's.
    np.testing.assert_array_equal(np.asarray(m.betas, np.float32), p["coefficients"])
    return m


def seeded_runtime(c, cls=None, **kw):
    from mcgb.core.runtime import Runtime
    cls = cls or Runtime
    rt = cls(make_model(c), int(c["L"]), list(c["T"]), seed=int(c["seed"]), **kw)
    np.testing.assert_array_equal(rt.betas.copy_to_host(), c["betas"] if "betas" in c else
                                  (1.0 / c["T"]).astype(np.float32))
    rt.state.copy_to_device(c["in"])
    return rt


@pytest.mark.parametrize("name", rc.RUNTIME_CASES)
def test_dropin_runtime_matches_reference_kernels(fx, name):
    from mcgb.device import device_array, to_device
    c = rc.case(fx, name)
    kw, cls = {}, None
    if name == "he3g_rt":
        from mcgb.models.he3.sampling import He3GaussianRuntime
        p = rc.params(c)
        cls, kw = He3GaussianRuntime, {"rho": float(p["rho"]), "proposal_mass": float(p["proposal_mass"])}
    rt = seeded_runtime(c, cls, **kw)
    for _ in range(int(c["sweeps"])):
        rt.sweep()
    rc.assert_rng_equal(rt.rng_states.copy_to_host(), c["rng_out"])
    rc.assert_states_close(rt.snapshot(), c["out"], c["kind"])
    if name == "he3g_rt":
        np.testing.assert_array_equal(rt.gaussian.counts.copy_to_host(), c["counts"])
        d = rt.sampling_diagnostics()
        for k in ("attempts", "accepted", "nonfinite_rejections"):
            np.testing.assert_array_equal(d[k], c[f"diag/{k}"], err_msg=k)
    # Measurements of the reference's final state, through the same calls.
    rt.state.copy_to_device(c["out"])
    rt.invalidate_energy_cache()
    fam = rc.family(c["kind"])
    rtol = rc.MEASURE_RTOL[fam]
    e = device_array(rt.R, np.float64)
    rt.measure_energy(e)
    np.testing.assert_allclose(e.copy_to_host(), c["energy"], rtol=rtol, atol=rtol)
    rt.invalidate_energy_cache()
    rc.assert_channels_close(rt.measure(), rc.channel(c, "measure"), rtol, name)
    got = rt.measure(temperature_indices=to_device(c["measure_order"]))
    rc.assert_channels_close(got, rc.channel(c, "measure_t"), rtol, name)


def run_dropin_pt(c):
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.simulation import Simulation
    rt = seeded_runtime(c)
    pt = ParallelTempering(rt, exchange_interval=int(c["interval"]), tracked_walkers=list(c["tracked"]),
                           history_stride=int(c["history_stride"]))
    res = Simulation(pt, thermalization_sweeps=int(c["thermalization"]),
                     measurement_sweeps=int(c["measurement"]), sample_interval=int(c["sample_interval"])).run()
    return rt, pt, res


def check_pt_result(c, res, name):
    fam = rc.family(c["kind"])
    meta = res["metadata"]
    np.testing.assert_array_equal(meta["sample_sweeps"], c["sample_sweeps"])
    rc.assert_channels_close(res["samples"], rc.channel(c, "samples"), rc.SAMPLE_RTOL[fam], name)
    d, ref = meta["parallel_tempering"], rc.channel(c, "pt")
    for k in rc.PT_EXACT:
        np.testing.assert_array_equal(np.asarray(d[k]), np.asarray(ref[k]), err_msg=k)
    np.testing.assert_array_equal(d["temperature_betas"], ref["temperature_betas"])
    np.testing.assert_allclose(d["acceptance_rates"], ref["acceptance_rates"], rtol=0, atol=0)
    return d, ref


@pytest.mark.parametrize("name", rc.PT_CASES)
def test_dropin_pt_simulation_matches_reference(fx, name):
    c = rc.case(fx, name)
    rt, pt, res = run_dropin_pt(c)
    d, ref = check_pt_result(c, res, name)
    for k in ("walker_ids", "sweeps", "exchange_rounds", "temperature_indices"):
        np.testing.assert_array_equal(d["walker_history"][k], ref[f"history/{k}"], err_msg=k)
    rc.assert_rng_equal(rt.rng_states.copy_to_host(), c["rng_out"])
    rc.assert_states_close(rt.snapshot(), c["out"], c["kind"])
    rc.assert_states_close(pt.snapshot(), c["out_t"], c["kind"])
    np.testing.assert_array_equal(rt.betas.copy_to_host(), c["betas_out"])


@pytest.mark.parametrize("split", [False, True])
def test_batched_ising_ladder_matches_reference_simulation(fx, split):
    """The batched engine (one launch per exchange window) reproduces the
    reference's Simulation(ParallelTempering(Runtime(IsingModel))) run bit
    for bit: samples, sample sweeps, maps, counters and the final lattice."""
    from mcgb.batch import LadderBatch
    from mcgb.models.ising.model import IsingModel
    c = rc.case(fx, "ising_pt")
    b = LadderBatch(IsingModel(J=float(rc.params(c)["J"])), [(int(c["L"]), list(c["T"]))], seeds=[int(c["seed"])],
                    exchange_interval=int(c["interval"]), exchange_seeds=[int(c["seed"]) + 1], cluster_size=2,
                    threads=64, initial_states=[c["in"]])
    if split:
        b.split_by_size(True)
    runs = b.simulate(thermalization_sweeps=int(c["thermalization"]), measurement_sweeps=int(c["measurement"]),
                      sample_interval=int(c["sample_interval"]))
    check_pt_result(c, runs[0], "ising_pt (batch)")
    np.testing.assert_array_equal(b.ladder_state(0), c["out"])
    rc.assert_rng_equal(b.ladder_rng(0), c["rng_out"])
