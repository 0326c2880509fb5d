"""Statistical parity: samplers that are not step-for-step identical to the
reference's must still sample the same distribution.

* XY, independent replicas: the batched engine with Gaussian proposals
  (mixed precision: float32 state, a (cos, sin) cache, fast intrinsics)
  against the reference's own path (the drop-in ``Runtime(XYModel())``,
  uniform delta = 1.5 proposals), 128 replicas per temperature; the errors
  come from the spread over independent replicas.
* XY, a parallel-tempering ladder: the batched engine against the drop-in
  ``Simulation(ParallelTempering(Runtime(XYModel())))``, and its energies
  against the plain float64 form of the same ladder.
* He3: the batched conditional-Gaussian sampler against the reference's
  Cartesian proposals through the drop-in runtime.
* Kawamura: the batched Gaussian sampler (theta and d Gaussian steps, the
  reference's tau flip) against the reference's uniform/flip/sphere
  proposals, on independent replicas and as parallel-tempering ladders.

Observables are the reference's analysis estimators with block-jackknife
errors (``stats.py``).  Each test compares m observable/temperature pairs;
every pair must agree within the Bonferroni bound that gives the whole test
the false-alarm rate of a single 3-sigma comparison (0.27 %): 3.51 sigma for
6 pairs, 3.79 for 18, 3.90 for 28.  The seeds are fixed, so each test is
deterministic.
"""

import numpy as np
import pytest

import stats

pytestmark = pytest.mark.gpu


def dropin_simulation(model, L, temps, seed, therm, meas, interval, pt=True):
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.core.simulation import Simulation
    rt = Runtime(model, L, temps, seed=seed)
    sim = ParallelTempering(rt, exchange_interval=10) if pt else rt
    return Simulation(sim, thermalization_sweeps=therm, measurement_sweeps=meas, sample_interval=interval).run()


def assert_agree(a, b):
    bound = stats.family_bound(stats.n_comparisons(a))
    bad = stats.compare(a, b, bound)
    assert not bad, (bound, bad)


def xy_replica_observables(samples, L, groups):
    """Energy per site, Binder cumulant and helicity modulus per temperature
    group, jackknifed over independent replicas (time means per replica)."""
    out = {"energy": ([], []), "binder": ([], []), "helicity": ([], [])}
    for T, idx in groups:
        m2 = samples["mx"][:, idx] ** 2 + samples["my"][:, idx] ** 2
        qx = samples["twist_sin_x"][:, idx]
        per = {"e": samples["energy"][:, idx].mean(0) / L ** 2, "m2": m2.mean(0), "m4": (m2 ** 2).mean(0),
               "cx": samples["twist_cos_x"][:, idx].mean(0), "qx": qx.mean(0), "qx2": (qx ** 2).mean(0)}

        def est(m, T=T):
            hel = (m["cx"] - (m["qx2"] - m["qx"] ** 2) / T) / L ** 2
            return np.stack((m["e"], 1 - m["m4"] / (2 * m["m2"] ** 2), hel))

        v, e = stats.jackknife(per, est, 1)
        for k, name in enumerate(out):
            out[name][0].append(v[k])
            out[name][1].append(e[k])
    return {k: (np.array(v), np.array(e)) for k, (v, e) in out.items()}


def test_xy_gaussian_batch_matches_reference_on_independent_replicas():
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    L, n = 16, 128
    temps = np.repeat([0.8, 1.0], n)
    groups = [(0.8, slice(0, n)), (1.0, slice(n, 2 * n))]
    therm, meas, interval = 3000, 40000, 10

    ref = dropin_simulation(XYModel(), L, temps, 42 + L, therm, meas, interval, pt=False)
    b = LadderBatch(XYModel(), [(L, temps)], seeds=[1042 + L], exchange_interval=None, proposal="gaussian")
    run = b.simulate(thermalization_sweeps=therm, measurement_sweeps=meas, sample_interval=interval)[0]

    a = xy_replica_observables(ref["samples"], L, groups)
    g = xy_replica_observables(run["samples"], L, groups)
    assert_agree(a, g)
    # Teeth: a 2e-3 shift of the energy per site would be several errors.
    assert np.all(a["energy"][1] < 4e-4) and np.all(g["energy"][1] < 4e-4)


def test_xy_gaussian_batch_and_plain_fp64_sample_the_reference_ladder():
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    from mcgb.plain64 import PlainXYLadder
    # Integrated autocorrelation times measured on these chains: at most 2
    # samples for the energy and helicity channels, 27 for the magnetisation
    # (Binder cumulant); blocks of 500 samples hold many of each.
    L, T = 16, np.geomspace(0.80, 1.30, 6)
    therm, meas, interval, block = 5000, 100000, 10, 500

    ref = dropin_simulation(XYModel(), L, T, 42 + L, therm, meas, interval)
    b = LadderBatch(XYModel(), [(L, T)], seeds=[1042 + L], exchange_interval=10, proposal="gaussian")
    run = b.simulate(thermalization_sweeps=therm, measurement_sweeps=meas, sample_interval=interval)[0]
    sigma = b.sigma_t.copy_to_host().astype(np.float64)
    acc = run["metadata"]["parallel_tempering"]["acceptance_rates"]
    assert np.all(acc > 0.05), acc

    a = stats.xy_observables(ref["samples"], L, T, block_size=block)
    g = stats.xy_observables(run["samples"], L, T, block_size=block)
    assert_agree(a, g)
    assert np.all(a["energy"][1] < 0.01) and np.ptp(a["energy"][0]) > 0.2

    plain = PlainXYLadder(L, T, 2042 + L, sigmas=sigma).simulate(therm, meas // 2, interval)
    p = stats.energy_observable(plain["samples"], L, block_size=block // 2)
    assert_agree({"energy": g["energy"]}, p)


def test_he3_conditional_gaussian_batch_samples_the_cartesian_distribution():
    from mcgb.batch import LadderBatch
    from mcgb.models.he3.model import He3Model
    # The reference's Cartesian chain decorrelates slowly: integrated
    # autocorrelation times up to 53 samples (Qzz alignment) and 39 (phase)
    # at the lowest temperature, against at most 2 for the Gaussian sampler.
    # Shorter runs underestimate its errors; blocks of 1000 samples do not.
    L, T = 8, np.geomspace(0.33, 0.47, 4)
    therm, meas, interval, block = 20000, 200000, 10, 1000

    ref = dropin_simulation(He3Model(), L, T, 42 + L, therm, meas, interval)
    b = LadderBatch(He3Model(), [(L, T)], seeds=[1042 + L], exchange_interval=10, gaussian=True,
                    rho=-0.9, proposal_mass=0.0)
    run = b.simulate(thermalization_sweeps=therm, measurement_sweeps=meas, sample_interval=interval)[0]

    a = stats.he3_observables(ref["samples"], L, T, block_size=block)
    g = stats.he3_observables(run["samples"], L, T, block_size=block)
    assert_agree(a, g)
    assert np.all(np.isfinite(a["energy"][1])) and np.all(a["energy"][1] > 0)


def test_kawamura_gaussian_batch_matches_reference_on_independent_replicas():
    """Gaussian theta/d proposals (batch) against the reference's uniform,
    flip and sphere proposals (drop-in Runtime): energy and the three order
    parameters of the Kawamura analysis, jackknifed over 96 independent
    replicas per temperature."""
    from mcgb.batch import LadderBatch
    from mcgb.models.kawamura.model import KawamuraModel
    L, n = 8, 96
    temps = np.repeat([0.6, 0.9], n)
    groups = [slice(0, n), slice(n, 2 * n)]
    therm, meas, interval = 2000, 20000, 10

    ref = dropin_simulation(KawamuraModel(), L, temps, 42 + L, therm, meas, interval, pt=False)
    b = LadderBatch(KawamuraModel(), [(L, temps)], seeds=[1042 + L], exchange_interval=None, proposal="gaussian",
                    sigma0=0.5)
    run = b.simulate(thermalization_sweeps=therm, measurement_sweeps=meas, sample_interval=interval)[0]

    def observables(samples):
        out = {k: ([], []) for k in ("energy", "chirality", "phase", "spin")}
        for idx in groups:
            per = {"e": samples["energy"][:, idx].mean(0) / L ** 2,
                   "tau2": (samples["chirality"][:, idx] ** 2).mean(0) / L ** 4,
                   "phase2": (samples["px"][:, idx] ** 2 + samples["py"][:, idx] ** 2).mean(0) / L ** 4,
                   "spin2": samples["spin2"][:, idx].mean(0) / L ** 4}
            v, e = stats.jackknife(per, lambda m: np.stack((m["e"], np.sqrt(m["tau2"]), np.sqrt(m["phase2"]),
                                                            np.sqrt(m["spin2"]))), 1)
            for k, name in enumerate(out):
                out[name][0].append(v[k])
                out[name][1].append(e[k])
        return {k: (np.array(v), np.array(e)) for k, (v, e) in out.items()}

    a, g = observables(ref["samples"]), observables(run["samples"])
    assert_agree(a, g)
    assert np.all(a["energy"][1] < 2e-3) and abs(a["energy"][0][0] - a["energy"][0][1]) > 0.1


def test_kawamura_gaussian_batch_samples_the_reference_distribution():
    from mcgb.batch import LadderBatch
    from mcgb.models.kawamura.model import KawamuraModel
    L, T = 8, np.geomspace(0.70, 1.00, 4)
    therm, meas, interval, block = 5000, 100000, 10, 500

    ref = dropin_simulation(KawamuraModel(), L, T, 42 + L, therm, meas, interval)
    b = LadderBatch(KawamuraModel(), [(L, T)], seeds=[1042 + L], exchange_interval=10, proposal="gaussian",
                    sigma0=0.5)
    run = b.simulate(thermalization_sweeps=therm, measurement_sweeps=meas, sample_interval=interval)[0]

    a = stats.kawamura_observables(ref["samples"], L, T, block_size=block)
    g = stats.kawamura_observables(run["samples"], L, T, block_size=block)
    assert_agree(a, g)
    # Teeth: the energy per site is resolved far below its spread over the
    # ladder (the reference chain is slowest near T = 0.79: error ~0.02).
    assert np.all(a["energy"][1] < 0.04) and np.ptp(a["energy"][0]) > 0.2
