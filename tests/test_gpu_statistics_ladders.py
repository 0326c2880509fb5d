"""Statistical parity at the shapes of the study, and of the PT swap rates.

* PT swap rates: the per-pair acceptance rates of the batched Gaussian XY
  ladder against the reference's path (Simulation(ParallelTempering(
  Runtime(XYModel()))), uniform delta = 1.5 proposals) -- the rates depend
  only on the equilibrium energy distributions, so any correct sampler gives
  the same ones -- jackknifed over independent ladders.
* The XY ladder the headline is quoted on (L = 128, 32 temperatures
  geometric in [0.70, 1.20], exchange every 10): the mixed-precision batch
  (float32, Gaussian widths tuned to ~50 %) against the plain float64 form
  (one lattice per launch, float64 state, proposals, exponentials and
  sums), energy, |m|, Binder cumulant and helicity modulus per temperature.
* A finite-size-scaling batch (sizes 16, 32, 64 in one ragged launch, 16
  temperatures with T = 0.893 among them): the same four observables per
  size and temperature against the plain float64 form, and the Binder
  crossings of successive sizes (utils/Analysis/crossings.py's method) where
  both forms see a unique one; the Ising batch reproduces the reference
  path's samples (same seeds), hence its Binder crossings, near the exact
  critical temperature.

Estimators are the reference's (tests/stats.py) with block-jackknife
errors; every comparison must hold within the Bonferroni bound that keeps
the whole test's false-alarm rate at one 3-sigma comparison.
"""

import numpy as np
import pytest

import stats

pytestmark = pytest.mark.gpu

TC_ISING = 2.0 / np.log(1.0 + np.sqrt(2.0))


def assert_agree(a, b):
    bound = stats.family_bound(stats.n_comparisons(a))
    bad = stats.compare(a, b, bound)
    assert not bad, (bound, bad)


def test_pt_swap_rates_batch_gaussian_vs_reference_proposals():
    from mcgb.batch import LadderBatch
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.core.simulation import Simulation
    from mcgb.models.xy.model import XYModel
    L, T, n, therm, meas = 16, np.geomspace(0.7, 1.2, 8), 12, 2000, 20000

    def rates(counts0, counts1):
        att, acc = counts1[0] - counts0[0], counts1[1] - counts0[1]
        return acc / att

    ref = []
    for k in range(n):
        rt = Runtime(XYModel(), L, T, seed=500 + k)
        pt = ParallelTempering(rt, exchange_interval=10)
        Simulation(pt, 0, therm, therm).run()
        d0 = pt.diagnostics()
        Simulation(pt, 0, meas, meas).run()
        d1 = pt.diagnostics()
        ref.append(rates((d0["attempts"], d0["accepted"]), (d1["attempts"], d1["accepted"])))
    b = LadderBatch(XYModel(), [(L, T)] * n, seeds=[900 + k for k in range(n)], exchange_interval=10,
                    proposal="gaussian")
    b.run(therm, tune=True)
    c0 = b.swap_counts.copy_to_host()
    b.run(meas)
    c1 = b.swap_counts.copy_to_host()
    got = [rates(c0[:, k * 7:(k + 1) * 7], c1[:, k * 7:(k + 1) * 7]) for k in range(n)]

    def over_ladders(x):
        x = np.asarray(x)
        return x.mean(0), x.std(0, ddof=1) / np.sqrt(len(x))
    a, g = {"swap_rate": over_ladders(ref)}, {"swap_rate": over_ladders(got)}
    assert_agree(a, g)
    # Teeth: rates well resolved and far from trivial.
    assert np.all(a["swap_rate"][1] < 0.02) and np.all((a["swap_rate"][0] > 0.1) & (a["swap_rate"][0] < 0.95))


def plain_and_batch(L_list, T, seeds, therm, meas, interval=10):
    """The batched Gaussian engine (one ragged launch over every size) and
    the plain float64 form with the batch's tuned widths, same schedule."""
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    from mcgb.plain64 import PlainXYLadder
    b = LadderBatch(XYModel(), [(L, T) for L in L_list], seeds=seeds, exchange_interval=interval,
                    proposal="gaussian")
    b.run(therm, tune=True)
    runs = b.simulate(thermalization_sweeps=0, measurement_sweeps=meas, sample_interval=interval)
    sig = b.sigma_t.copy_to_host().astype(np.float64)
    plain = []
    for k, L in enumerate(L_list):
        ladder = PlainXYLadder(L, T, seeds[k] + 7919, sigmas=sig[k * len(T):(k + 1) * len(T)],
                               exchange_interval=interval)
        plain.append(ladder.simulate(therm, meas, interval))
    return runs, plain


def test_xy_headline_ladder_mixed_batch_vs_plain_fp64():
    L, T = 128, np.geomspace(0.70, 1.20, 32)
    runs, plain = plain_and_batch([L], T, [42 + L], therm=5000, meas=20000)
    a = stats.xy_observables(plain[0]["samples"], L, T, block_size=200)
    g = stats.xy_observables(runs[0]["samples"], L, T, block_size=200)
    assert_agree(a, g)
    # Teeth: energy and helicity per site resolved to well under their spread.
    assert np.all(a["energy"][1] < 2e-3) and np.ptp(a["energy"][0]) > 0.3
    assert np.ptp(a["helicity"][0]) > 0.3


def test_xy_fss_batch_vs_plain_fp64_and_binder_crossings():
    Ls = [16, 32, 64]
    T = np.sort(np.append(np.geomspace(0.78, 1.02, 15), 0.893))
    runs, plain = plain_and_batch(Ls, T, [42 + L for L in Ls], therm=3000, meas=15000)
    a, g = {}, {}
    for k, L in enumerate(Ls):
        oa = stats.xy_observables(plain[k]["samples"], L, T, block_size=200)
        og = stats.xy_observables(runs[k]["samples"], L, T, block_size=200)
        for name in oa:
            a[f"{name}_L{L}"], g[f"{name}_L{L}"] = oa[name], og[name]
    assert_agree(a, g)
    i893 = int(np.argmin(np.abs(T - 0.893)))
    for L in Ls:   # the helicity modulus at T = 0.893 is resolved
        assert a[f"helicity_L{L}"][1][i893] < 0.05

    def binder(m):
        return 1 - m["m4"] / (2 * m["m2"] ** 2)

    def m2(run, L):
        s = run["samples"]
        return {"m2": (np.asarray(s["mx"]) ** 2 + np.asarray(s["my"]) ** 2) / L ** 4}
    for (k1, L1), (k2, L2) in ((0, 16), (1, 32)), ((1, 32), (2, 64)):
        ca = stats.binder_crossing(m2(plain[k1], L1), m2(plain[k2], L2), T, binder, 200)
        cg = stats.binder_crossing(m2(runs[k1], L1), m2(runs[k2], L2), T, binder, 200)
        if ca is not None and cg is not None:
            bound = stats.family_bound(2)
            assert abs(ca[0] - cg[0]) <= bound * np.hypot(ca[1], cg[1]), (L1, L2, ca, cg)


def test_ising_fss_batch_reproduces_the_reference_path_and_its_crossings():
    """The finite-size-scaling batch of three sizes (one ragged launch per
    window) against the reference's path, one
    Simulation(ParallelTempering(Runtime(IsingModel()))) per size with the
    same seeds: Ising is integer work, so every sample is identical and so
    are the Binder crossings of L = 16/32 and 32/64 computed from them
    (utils/Analysis/crossings.py's method, jackknife errors); both crossings
    lie near Tc (small sizes on a 16-point ladder carry finite-size and
    interpolation shifts of order 0.01)."""
    from mcgb.batch import LadderBatch
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.core.simulation import Simulation
    from mcgb.models.ising.model import IsingModel
    Ls = [16, 32, 64]
    T = np.geomspace(2.1, 2.45, 16)
    therm, meas, every, block = 5000, 40000, 10, 400
    b = LadderBatch(IsingModel(), [(L, T) for L in Ls], seeds=[42 + L for L in Ls], exchange_interval=10)
    runs = b.simulate(thermalization_sweeps=therm, measurement_sweeps=meas, sample_interval=every)
    ref = []
    for L in Ls:
        pt = ParallelTempering(Runtime(IsingModel(), L, T, seed=42 + L), exchange_interval=10)
        ref.append(Simulation(pt, therm, meas, every).run())
    for k in range(3):
        for name in ("energy", "magnetization"):
            np.testing.assert_array_equal(runs[k]["samples"][name], ref[k]["samples"][name], err_msg=name)

    def binder(m):
        return 1 - m["m4"] / (3 * m["m2"] ** 2)

    def m2(run, L):
        return {"m2": (np.asarray(run["samples"]["magnetization"], np.float64) / L ** 2) ** 2}
    for (k1, L1), (k2, L2) in ((0, 16), (1, 32)), ((1, 32), (2, 64)):
        cg = stats.binder_crossing(m2(runs[k1], L1), m2(runs[k2], L2), T, binder, block)
        ca = stats.binder_crossing(m2(ref[k1], L1), m2(ref[k2], L2), T, binder, block)
        assert cg is not None and cg == ca, (L1, L2, cg, ca)
        assert abs(cg[0] - TC_ISING) < 0.03 and cg[1] < 0.01, (L1, L2, cg)
