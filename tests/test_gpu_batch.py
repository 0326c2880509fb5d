"""Batched ladder engine against the per-colour drop-in path and the oracle."""

import contextlib
from unittest.mock import patch

import numpy as np
import pytest

import npref
import oracle

pytestmark = pytest.mark.gpu


def dropin_ising(L, temps, seed, init):
    from mcgb.core.runtime import Runtime
    from mcgb.models.ising.model import IsingModel
    rt = Runtime(IsingModel(J=1.0), L, temps, seed=seed)
    rt.state.copy_to_device(init)
    return rt


def seeded_spins(rng, R, L):
    return rng.choice(np.array([-1, 1], dtype=np.int8), (R, L, L))


@pytest.mark.parametrize("cluster_size,threads", [(1, 256), (2, 512), (4, 1024), (8, 128), (2, 96), (1, 288)])
def test_ising_batch_bit_exact_with_dropin_runtime(cluster_size, threads):
    from mcgb.batch import LadderBatch
    from mcgb.models.ising.model import IsingModel
    L, temps = 64, [1.5, 2.269, 3.0]
    rng = np.random.default_rng(106)
    inits = [seeded_spins(rng, 1, L) for _ in temps]
    b = LadderBatch(IsingModel(), [(L, [T]) for T in temps], seeds=[42 + L] * 3, exchange_interval=None,
                    cluster_size=cluster_size, threads=threads, initial_states=inits)
    b.run(100)
    for k, T in enumerate(temps):
        rt = dropin_ising(L, [T], 42 + L, inits[k])
        for _ in range(100):
            rt.sweep()
        np.testing.assert_array_equal(b.ladder_state(k), rt.snapshot())
        rs = rt.rng_states.copy_to_host()
        np.testing.assert_array_equal(b.ladder_rng(k), np.stack([rs["s0"], rs["s1"]], axis=1))
    e = b.energies.copy_to_host()
    for k in range(3):
        np.testing.assert_array_equal(e[k], oracle.ising_energy(b.ladder_state(k), np.float32(1))[0])


@pytest.mark.parametrize("L2,split", [(16, False), (24, True), (64, False), (64, True)])
def test_ising_batch_pt_simulation_equals_dropin_simulation(L2, split):
    """Same seeds: identical samples, maps and swap counters to Simulation(ParallelTempering),
    also with the ladders of two sizes run as one launch per size.  The 64^2
    ladder's strips (512-byte colour rows, 16-byte aligned) arrive by bulk
    copies in the fused launches; the 16^2 and 24^2 ones by per-thread loads."""
    from mcgb.batch import LadderBatch
    from mcgb.core.parallel_tempering import ParallelTempering
    from mcgb.core.runtime import Runtime
    from mcgb.core.simulation import Simulation
    from mcgb.models.ising.model import IsingModel
    L, temps = 16, np.geomspace(1.8, 3.0, 5)
    init = seeded_spins(np.random.default_rng(5), 5, L)
    init2 = seeded_spins(np.random.default_rng(6), 4, L2)
    b = LadderBatch(IsingModel(), [(L, temps), (L2, temps[:4])], seeds=[58, 77], exchange_interval=3,
                    exchange_seeds=[59, 78], cluster_size=2, threads=128,
                    initial_states=[init, init2])
    if split:
        b.split_by_size(True)
        assert len(b.groups) == 2
    runs = b.simulate(thermalization_sweeps=7, measurement_sweeps=40, sample_interval=2)
    for k, (Lk, init_k, T_k, seed) in enumerate(((L, init, temps, 58), (L2, init2, temps[:4], 77))):
        rt = Runtime(IsingModel(), Lk, T_k, seed=seed)
        rt.state.copy_to_device(init_k)
        pt = ParallelTempering(rt, exchange_interval=3, seed=seed + 1)
        ref = Simulation(pt, thermalization_sweeps=7, measurement_sweeps=40, sample_interval=2).run()
        for name in ref["samples"]:
            np.testing.assert_array_equal(runs[k]["samples"][name], ref["samples"][name], err_msg=name)
        np.testing.assert_array_equal(runs[k]["metadata"]["sample_sweeps"], ref["metadata"]["sample_sweeps"])
        d, dr = runs[k]["metadata"]["parallel_tempering"], ref["metadata"]["parallel_tempering"]
        for key in ("attempts", "accepted", "walker_to_temperature", "temperature_to_walker",
                    "walker_round_trips", "walker_round_trip_total_sweeps", "exchange_rounds", "sweeps"):
            np.testing.assert_array_equal(d[key], dr[key], err_msg=key)
        np.testing.assert_array_equal(b.ladder_state(k), rt.snapshot())


@pytest.mark.parametrize("resident,split", [(True, False), (False, False), (True, True), (False, True),
                                            (True, "side"), (False, "side")])
def test_graph_replay_equals_direct_launches(resident, split):
    """Replayed graphs (resident: ten windows per launch, each walker waiting
    for its own pair only; split: one launch per lattice size, each with its
    own cluster shape, the last advancing the clock; "side": the per-size
    launches side by side on streams of their own, each advancing its own
    copy of the clock, never resident) against one fused launch per window
    over the whole batch, on ragged ladders with unpaired end slots and a
    two-slot ladder: identical chains, maps, betas, swap and round-trip
    counters, samples and clock."""
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    ladders = [(32, np.geomspace(0.7, 1.2, 6)), (16, [0.8, 1.0]), (16, [0.7, 0.9, 1.1])]
    kw = dict(seeds=[3, 4, 5], exchange_interval=5, proposal="gaussian", cluster_size=2, threads=256)
    a = LadderBatch(XYModel(), ladders, resident=resident, **kw)
    c = LadderBatch(XYModel(), ladders, resident=False, **kw)
    if split:
        a.split_by_size(True, concurrent=split == "side")
        assert [sizes for sizes, *_ in a.shapes()] == [[16], [32]]
    assert a.resident == (resident and split != "side")
    for b in (a, c):
        b.allocate_samples(5, 5, 12)
    a.run(60, graph=True)
    c.run(60, graph=False)
    a.check_errors()
    for k in range(len(ladders)):
        np.testing.assert_array_equal(a.ladder_state(k), c.ladder_state(k))
    for name in ("w2t", "t2w", "betas", "swap_counts", "trips", "energies", "clock", "samples"):
        np.testing.assert_array_equal(getattr(a, name).copy_to_host(), getattr(c, name).copy_to_host(),
                                      err_msg=name)
    np.testing.assert_array_equal(a.clock.copy_to_host(), [60, 12])
    w2t, t2w = a.w2t.copy_to_host(), a.t2w.copy_to_host()
    for s0, n in ((0, 6), (6, 2), (8, 3)):
        np.testing.assert_array_equal(t2w[s0 + w2t[s0:s0 + n]], np.arange(n))
    # 12 rounds: the 6-slot ladder alternates 3 and 2 pairs, the others 1
    assert a.swap_counts.copy_to_host()[0].sum() == 6 * 3 + 6 * 2 + 12 + 12


@pytest.mark.parametrize("proposal,L,cluster_size,threads",
                         [("uniform", 32, 4, 128), ("gaussian", 32, 4, 128), ("gaussian", 64, 1, 96),
                          ("gaussian", 128, 1, 1024), ("gaussian", 512, 16, 1024)])
def test_xy_batch_window_matches_oracle(proposal, L, cluster_size, threads):
    """One 1-sweep window per colour order against the oracle: RNG bit-exact,
    angles within float32 rounding except rare acceptance flips; streams in
    registers (L=32), in global memory two visits at a time (L=64) and one
    at a time (L=128, and L=512 on 16 CTAs: four plaquettes a thread)."""
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    temps = np.array([0.7, 0.9, 1.1, 1.2])
    init = np.random.default_rng(6).uniform(-np.pi, np.pi, (4, L, L)).astype(np.float32)
    b = LadderBatch(XYModel(), [(L, temps)], seeds=[5], exchange_interval=None, proposal=proposal,
                    sigma0=1.1, cluster_size=cluster_size, threads=threads, initial_states=[init])
    b.run(1)
    ref, rr = init.copy(), oracle.rng_states(4 * L * L, 5)
    betas = (1 / temps).astype(np.float32)
    for c in range(4):
        if proposal == "uniform":
            oracle.xy_update_color(ref, rr, betas, c, np.float32(1), np.float32(1.5))
        else:
            oracle.xy_update_color_gauss(ref, rr, betas, np.full(4, 1.1, np.float32), c, np.float32(1))
    np.testing.assert_array_equal(b.ladder_rng(0), rr)
    got = b.ladder_state(0)
    d = np.abs(np.angle(np.exp(1j * (got.astype(np.float64) - ref))))
    assert np.mean(d > 1e-4) <= 1e-3


def test_xy_running_energy_tracks_fp64_recompute():
    """Single-sweep energy differences agree with an FP64 recompute within 1e-5 relative."""
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    L, temps = 64, np.geomspace(0.7, 1.2, 8)
    init = np.random.default_rng(9).uniform(-np.pi, np.pi, (8, L, L)).astype(np.float32)
    b = LadderBatch(XYModel(), [(L, temps)], exchange_interval=1, proposal="gaussian", initial_states=[init])
    e0 = oracle.xy_energy(init, np.float32(1))
    np.testing.assert_allclose(b.energies.copy_to_host(), e0, rtol=1e-12)
    b.run(1)
    after = b.ladder_state(0)
    e1_exact = oracle.xy_energy(after, np.float32(1))
    e1_run = b.energies.copy_to_host()
    d_run, d_exact = e1_run - e0, e1_exact - e0
    assert np.all(np.abs(d_run - d_exact) <= 1e-5 * np.abs(d_exact))
    b.run(200)
    e_run = b.energies.copy_to_host()
    drift = b.recompute_energy().copy_to_host()
    exact = oracle.xy_energy(b.ladder_state(0), np.float32(1))
    np.testing.assert_allclose(b.energies.copy_to_host(), exact, rtol=1e-10)
    assert np.all(np.abs(drift) <= 1e-5 * np.abs(exact))
    np.testing.assert_allclose(e_run - drift, exact, rtol=1e-10)


def test_xy_batch_samples_match_exact_observables():
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    L, temps = 32, np.geomspace(0.7, 1.2, 4)
    b = LadderBatch(XYModel(), [(L, temps)], exchange_interval=4, proposal="gaussian", cluster_size=2,
                    threads=256)
    runs = b.simulate(thermalization_sweeps=10, measurement_sweeps=8, sample_interval=8)
    last = {k: v[-1] for k, v in runs[0]["samples"].items()}
    state = b.ladder_state(0)
    ref = npref.xy(state, 1.0)
    order = b.w2t.copy_to_host()
    for name in ref:
        got = np.empty(4)
        got[order] = ref[name]
        np.testing.assert_allclose(last[name], got, rtol=1e-5, atol=2e-3 * L, err_msg=name)


def _mixed_size_batch(model, ladders, seeds, inits, clusters, shape, **kw):
    """One group whose clusters each run a work list of several lattice
    sizes (at most `clusters` clusters), a sample on every window's last
    sweep."""
    from mcgb.batch import LadderBatch
    cap = patch.object(LadderBatch, "max_clusters", lambda self, C, T, idx=None: clusters)
    with cap if clusters else contextlib.nullcontext():
        b = LadderBatch(model, ladders, seeds=seeds, exchange_interval=5, initial_states=inits, **kw)
        b.split_by_size(False)
        b.configure(*shape)
    b.allocate_samples(5, 5, 16)
    return b


def test_mixed_size_work_lists_with_window_end_samples_are_exact():
    """A cluster whose work list holds several sizes, with the window-end
    sample carrying the epilogue: bit-identical to one replica per cluster."""
    from mcgb.models.ising.model import IsingModel
    rng = np.random.default_rng(8)
    ladders = [(L, list(np.geomspace(2.0, 2.6, 8))) for L in (16, 32, 48)]
    seeds = [5, 6, 7]
    inits = [seeded_spins(rng, 8, L) for L, _ in ladders]
    mixed = _mixed_size_batch(IsingModel(), ladders, seeds, inits, 2, (2, 128))
    assert mixed.n_clusters == 2 and not mixed.resident
    wp, wi = mixed.work_ptr.copy_to_host(), mixed.work_idx.copy_to_host()
    assert all(len(set(mixed.table_host["L"][wi[wp[c]:wp[c + 1]]])) > 1 for c in range(2))
    one = _mixed_size_batch(IsingModel(), ladders, seeds, inits, None, (2, 128))
    assert one.n_clusters == 24
    for b in (mixed, one):
        b.run(40)
        b.check_errors()
    for k in range(3):
        np.testing.assert_array_equal(mixed.ladder_state(k), one.ladder_state(k))
    np.testing.assert_array_equal(mixed.w2t.copy_to_host(), one.w2t.copy_to_host())
    np.testing.assert_array_equal(mixed.samples.copy_to_host(), one.samples.copy_to_host())
    np.testing.assert_array_equal(mixed.energies.copy_to_host(), one.energies.copy_to_host())
    assert np.all(mixed.recompute_energy().copy_to_host() == 0.0)


def test_he3_mixed_size_work_lists_keep_the_running_energy():
    """He3 (float state, running float energy) on mixed-size work lists with
    window-end samples: the running energy stays within rounding of an FP64
    recompute of the state."""
    from mcgb.models.he3.model import He3Model
    T = list(np.geomspace(0.33, 0.47, 6))
    ladders = [(L, T) for L in (32, 48, 64)]
    b = _mixed_size_batch(He3Model(), ladders, [1, 2, 3], None, 2, (2, 256), gaussian=True)
    b.run(60)
    b.check_errors()
    drift = b.recompute_energy().copy_to_host()
    scale = np.maximum(np.abs(b.energies.copy_to_host()), b.table_host["L"].astype(np.float64) ** 2)
    assert np.max(np.abs(drift) / scale) < 1e-5


def test_ragged_batch_ladders_match_their_own_runtimes():
    from mcgb.batch import LadderBatch
    from mcgb.models.ising.model import IsingModel
    ladders = [(16, [2.0, 2.5]), (32, [2.0, 2.5]), (64, [2.2, 2.6])]
    rng = np.random.default_rng(1)
    inits = [seeded_spins(rng, 2, L) for L, _ in ladders]
    b = LadderBatch(IsingModel(), ladders, seeds=[10, 20, 30], exchange_interval=None, initial_states=inits)
    assert b.cluster_size in (1, 2, 4, 8)
    b.run(30)
    for k, (L, T) in enumerate(ladders):
        rt = dropin_ising(L, T, [10, 20, 30][k], inits[k])
        for _ in range(30):
            rt.sweep()
        np.testing.assert_array_equal(b.ladder_state(k), rt.snapshot())


def test_invalid_batches_raise():
    from mcgb.batch import LadderBatch
    from mcgb.models.ising.model import IsingModel
    with pytest.raises(ValueError):
        LadderBatch(IsingModel(), [(6, [1.0, 1.0])])
    with pytest.raises(ValueError):
        LadderBatch(IsingModel(), [(16, [2.0])], exchange_interval=10)
    with pytest.raises(ValueError):
        LadderBatch(IsingModel(), [(16, [2.0, 3.0])], cluster_size=17, threads=128)


def test_effective_cluster_serves_lattices_smaller_than_the_cluster():
    """L=12 in clusters of 16 CTAs: 6 plaquette rows -> 6 CTAs hold it, 10 idle."""
    from mcgb.batch import LadderBatch
    from mcgb.models.ising.model import IsingModel
    ladders = [(12, [2.0, 2.5]), (64, [2.0, 2.5]), (10, [2.2, 2.3])]
    rng = np.random.default_rng(12)
    inits = [seeded_spins(rng, 2, L) for L, _ in ladders]
    b = LadderBatch(IsingModel(), ladders, seeds=[1, 2, 3], exchange_interval=None, cluster_size=16,
                    threads=128, initial_states=inits)
    assert [b.effective_cluster(L, 16) for L, _ in ladders] == [6, 16, 5]
    b.run(9)
    for k, (L, T) in enumerate(ladders):
        rt = dropin_ising(L, T, [1, 2, 3][k], inits[k])
        for _ in range(9):
            rt.sweep()
        np.testing.assert_array_equal(b.ladder_state(k), rt.snapshot())


# ------------------------------------------------------------ Kawamura and He3

def assert_close_sites(got, ref, axes, tol=1e-4, max_frac=2e-3):
    d = np.abs(got.astype(np.complex128) - ref.astype(np.complex128))
    if axes:
        d = d.max(axis=axes)
    assert np.mean(d > tol) <= max_frac, f"{int(np.sum(d > tol))} of {d.size} sites differ"


def test_kawamura_batch_sweep_matches_oracle_and_tracks_energy():
    from mcgb.batch import LadderBatch
    from mcgb.models.kawamura.model import KawamuraModel
    L, temps = 32, np.linspace(0.65, 0.8, 4)
    init = npref.random_kawamura(np.random.default_rng(9), 4, L)
    b = LadderBatch(KawamuraModel(), [(L, temps)], seeds=[8], exchange_interval=None, cluster_size=2,
                    threads=256, initial_states=[init])
    e0 = b.energies.copy_to_host()
    np.testing.assert_allclose(e0, npref.kawamura(init, 1.0)["energy"], rtol=1e-10, atol=1e-9)
    b.run(1)
    ref, rr = init.copy(), oracle.rng_states(4 * L * L, 8)
    betas = (1 / temps).astype(np.float32)
    for c in range(4):
        oracle.kawamura_update_color(ref, rr, betas, c, np.float32(1), np.float32(1.5))
    np.testing.assert_array_equal(b.ladder_rng(0), rr)
    got = b.ladder_state(0)
    assert_close_sites(got, ref, -1)
    d_run = b.energies.copy_to_host() - e0
    d_exact = npref.kawamura(got, 1.0)["energy"] - e0
    assert np.all(np.abs(d_run - d_exact) <= 1e-5 * np.abs(d_exact))
    b.run(40)
    drift = b.recompute_energy().copy_to_host()
    assert np.all(np.abs(drift) <= 1e-5 * np.abs(b.energies.copy_to_host()))
    st = b.ladder_state(0)
    np.testing.assert_allclose(np.linalg.norm(st[..., 2:], axis=-1), 1, atol=3e-6)
    assert set(np.unique(st[..., 1])) <= {-1.0, 1.0}


@pytest.mark.parametrize("L,cluster_size,threads", [(32, 2, 256), (32, 1, 64), (96, 2, 512)])
def test_kawamura_gaussian_batch_sweep_matches_oracle(L, cluster_size, threads):
    """Gaussian proposals (theta and d) against the oracle's restatement:
    streams bit-exact (five draws per visit), sites within float32 rounding;
    streams in registers, in global memory two visits at a time (64
    threads) and one at a time (512)."""
    from mcgb.batch import LadderBatch
    from mcgb.models.kawamura.model import KawamuraModel
    temps = np.linspace(0.65, 0.8, 4)
    init = npref.random_kawamura(np.random.default_rng(19), 4, L)
    sig = np.array([0.5, 0.6, 0.7, 0.8], np.float32)
    b = LadderBatch(KawamuraModel(), [(L, temps)], seeds=[18], exchange_interval=None, proposal="gaussian",
                    cluster_size=cluster_size, threads=threads, initial_states=[init])
    b.sigma_t.copy_to_device(sig)
    e0 = b.energies.copy_to_host()
    b.run(2)
    ref, rr = init.copy(), oracle.rng_states(4 * L * L, 18)
    oracle.kawamura_sweeps_gauss(ref, rr, (1 / temps).astype(np.float32), sig, np.float32(1), 2)
    np.testing.assert_array_equal(b.ladder_rng(0), rr)
    got = b.ladder_state(0)
    assert_close_sites(got, ref, -1)
    d_run = b.energies.copy_to_host() - e0
    d_exact = npref.kawamura(got, 1.0)["energy"] - e0
    assert np.all(np.abs(d_run - d_exact) <= 1e-5 * np.abs(d_exact))
    np.testing.assert_allclose(np.linalg.norm(got[..., 2:], axis=-1), 1, atol=3e-6)


def test_kawamura_batch_pt_samples_match_numpy():
    from mcgb.batch import LadderBatch
    from mcgb.models.kawamura.model import KawamuraModel
    L, temps = 16, np.linspace(0.65, 0.8, 5)
    b = LadderBatch(KawamuraModel(J=1.1), [(L, temps), (32, temps[:3])], exchange_interval=3, cluster_size=2,
                    threads=128)
    runs = b.simulate(thermalization_sweeps=5, measurement_sweeps=12, sample_interval=6)
    for k, (Lk, Tk) in enumerate(b.ladders):
        last = {name: v[-1] for name, v in runs[k]["samples"].items()}
        st = b.ladder_state(k)
        ref = npref.kawamura(st, 1.1)
        order = b.w2t.copy_to_host()[b.ladder_starts_host[k]:b.ladder_starts_host[k] + len(Tk)]
        for name in ref:
            want = np.empty(len(Tk))
            want[order] = ref[name]
            np.testing.assert_allclose(last[name], want, rtol=1e-5, atol=2e-3 * Lk * Lk ** 0.5, err_msg=name)
        assert sum(runs[k]["metadata"]["parallel_tempering"]["attempts"]) > 0


@pytest.mark.parametrize("gaussian", [False, True])
def test_he3_batch_sweep_matches_oracle_and_tracks_energy(gaussian):
    from mcgb.batch import LadderBatch
    from mcgb.models.he3.model import He3Model
    L, temps = 16, np.array([0.3, 0.4, 0.6])
    model = He3Model(pressure=20, g_d=0.001)
    init = npref.random_he3(np.random.default_rng(4), (3, L, L, 3, 2))
    b = LadderBatch(model, [(L, temps)], seeds=[227], exchange_interval=None, gaussian=gaussian,
                    cluster_size=2, threads=128, initial_states=[init])
    e0 = b.energies.copy_to_host()
    np.testing.assert_allclose(e0, npref.he3_energy(init, float(model.K), model.betas, g_d=float(model.g_d)),
                               rtol=1e-9, atol=1e-9)
    b.run(1)
    ref, rr = init.copy(), oracle.rng_states(3 * L * L, 227)
    betas = (1 / temps).astype(np.float32)
    counts = np.zeros((3, 3, L, L), np.int64)
    for c in range(4):
        if gaussian:
            oracle.he3_gaussian_update_color(ref, rr, betas, c, model.betas, model.K, np.float32(-0.9),
                                             np.float32(0), model.g_d, counts)
        else:
            oracle.he3_update_color(ref, rr, betas, c, model.betas, model.K, model.delta, model.g_d)
    np.testing.assert_array_equal(b.ladder_rng(0), rr)
    got = b.ladder_state(0)
    assert_close_sites(got, ref, (-2, -1))
    d_run = b.energies.copy_to_host() - e0
    d_exact = npref.he3_energy(got, float(model.K), model.betas, g_d=float(model.g_d)) - e0
    assert np.all(np.abs(d_run - d_exact) <= 1e-5 * np.abs(d_exact) + 1e-4)
    b.run(20)
    drift = b.recompute_energy().copy_to_host()
    assert np.all(np.abs(drift) <= 1e-5 * np.maximum(np.abs(b.energies.copy_to_host()), L * L))
    if gaussian:
        d = b.sampling_diagnostics()
        assert sum(d["nonfinite_rejections"]) == 0 and 0 < sum(d["accepted"]) < sum(d["attempts"])


def test_he3_ragged_batch_samples_match_numpy():
    from mcgb.batch import LadderBatch
    from mcgb.models.he3.model import He3Model
    model = He3Model(pressure=20)
    ladders = [(16, [0.33, 0.4, 0.47]), (32, [0.33, 0.4, 0.47])]
    b = LadderBatch(model, ladders, exchange_interval=2, gaussian=True)
    runs = b.simulate(thermalization_sweeps=4, measurement_sweeps=6, sample_interval=6)
    for k, (Lk, Tk) in enumerate(b.ladders):
        last = {name: v[-1] for name, v in runs[k]["samples"].items()}
        st = b.ladder_state(k)
        ref = npref.he3(st, float(model.K), model.betas)
        order = b.w2t.copy_to_host()[b.ladder_starts_host[k]:b.ladder_starts_host[k] + len(Tk)]
        for name in ref:
            want = np.empty(len(Tk))
            want[order] = ref[name]
            np.testing.assert_allclose(last[name], want, rtol=2e-5, atol=1e-3 * Lk, err_msg=name)


@pytest.mark.parametrize("L,cluster_size,threads", [(64, 1, 128), (64, 1, 96), (128, 1, 1024), (512, 2, 1024),
                                                    (512, 16, 1024)])
def test_streams_in_global_memory_path_is_bit_exact(L, cluster_size, threads):
    """Strips with more plaquettes than two per thread keep the RNG streams in
    global memory (the large-L path): two visits in flight at <= 512 threads
    (an odd count per thread at 96), one at 1024; Ising stays bit-identical,
    up to the largest lattice of the finite-size batch (L=512, 16 and 2 CTAs
    a replica: 4 and 32 plaquettes a thread per colour)."""
    from mcgb.batch import LadderBatch
    from mcgb.models.ising.model import IsingModel
    temps = [2.0, 2.4]
    init = seeded_spins(np.random.default_rng(3), 2, L)
    b = LadderBatch(IsingModel(), [(L, temps)], seeds=[99], exchange_interval=None, cluster_size=cluster_size,
                    threads=threads, initial_states=[init])
    b.run(12)
    rt = dropin_ising(L, temps, 99, init)
    for _ in range(12):
        rt.sweep()
    np.testing.assert_array_equal(b.ladder_state(0), rt.snapshot())


def test_simulated_ladders_save_load_and_summarise(tmp_path):
    """LadderBatch.simulate -> run file (reference format) -> PT summary."""
    from mcgb import ladder, pt_analysis, runs
    from mcgb.batch import LadderBatch
    from mcgb.models.ising.model import IsingModel
    ladders = ladder.ragged_ladders([8, 16], 2.0, 2.6, 6, Tc=2.269, tc_window=0.2, tc_fraction=0.5)
    b = LadderBatch(IsingModel(), ladders, exchange_interval=5)
    out = runs.runs_by_size(b.simulate(thermalization_sweeps=50, measurement_sweeps=200, sample_interval=10))
    runs.save_runs(tmp_path / "fss.npz", out)
    back = runs.load_runs(tmp_path / "fss.npz")
    assert sorted(back) == [8, 16]
    for L in (8, 16):
        for name, values in out[L]["samples"].items():
            np.testing.assert_array_equal(back[L]["samples"][name], values)
        assert back[L]["samples"]["energy"].shape == (20, 6)
    s = pt_analysis.pt_summary(back)
    for L in (8, 16):
        # 250 sweeps, an exchange every 5: 50 rounds of 3 and 2 pairs alternately.
        assert sum(s[L]["attempts"]) == 25 * 3 + 25 * 2
        assert 0 < s[L]["aggregate_acceptance"] <= 1
        assert s[L]["temperatures"] == pytest.approx(list(ladders[0][1]))


def test_host_round_trip_resumes_the_chain_exactly():
    """download_state/upload_state move the chain state (angles, streams,
    running energies; the (cos, sin) cache is rebuilt from the angles on the
    device, bit for bit what the sweeps left): resuming from the host copy
    repeats the same sweeps bit for bit; a state-only upload also rebuilds the
    energies."""
    import torch
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    L, T = 32, np.geomspace(0.8, 1.2, 4)
    init = np.random.default_rng(12).uniform(-np.pi, np.pi, (4, L, L)).astype(np.float32)
    b = LadderBatch(XYModel(), [(L, T)], exchange_interval=None, proposal="gaussian", initial_states=[init])
    b.run(30)
    evolved = b.aux.copy_to_host()
    b.refresh_aux()
    np.testing.assert_array_equal(b.aux.copy_to_host().view(np.uint32), evolved.view(np.uint32))
    host = b.pinned_state_buffers()
    assert set(host) == {"chain"} and host["chain"].numel() >= b.state.nbytes + b.rng.nbytes + b.e_run.nbytes
    assert host["chain"].numel() < b.state.nbytes + b.rng.nbytes + b.aux.nbytes
    b.download_state(host)
    torch.cuda.synchronize()
    b.run(20)
    first = (b.ladder_state(0), b.ladder_rng(0), b.energies.copy_to_host())
    b.upload_state(host)
    b.run(20)
    again = (b.ladder_state(0), b.ladder_rng(0), b.energies.copy_to_host())
    for x, y in zip(first, again):
        np.testing.assert_array_equal(np.asarray(x).view(np.uint8), np.asarray(y).view(np.uint8))
    state_bytes = b.state.raw().cpu().clone()
    rng_bytes = b.rng.raw().cpu().clone()
    b.upload_state({"state": state_bytes, "rng": rng_bytes})
    drift = b.recompute_energy().copy_to_host()
    assert np.all(np.abs(drift) < 1e-6 * L * L)


@pytest.mark.parametrize("proposal", ["uniform", "gaussian"])
def test_kawamura_cache_is_a_function_of_the_angles(proposal):
    """The Kawamura (cos, sin) cache after sweeps equals its rebuild from the
    angles bit for bit, so host round trips need not carry it."""
    from mcgb.batch import LadderBatch
    from mcgb.models.kawamura.model import KawamuraModel
    b = LadderBatch(KawamuraModel(), [(16, np.geomspace(0.8, 1.2, 4))], exchange_interval=None,
                    proposal=proposal, cluster_size=2, threads=128)
    b.run(25)
    evolved = b.aux.copy_to_host()
    b.refresh_aux()
    np.testing.assert_array_equal(b.aux.copy_to_host().view(np.uint32), evolved.view(np.uint32))


def test_resident_wait_that_runs_out_is_reported_and_the_batch_recovers():
    """Failure detection: with a wait limit of zero polls every walker of a
    resident launch that waits for its pair's decision gives up at once; the
    kernel raises its error flag and returns (no hang), check_errors()
    reports it as MCGBTimeout, rebuilds consistent slot maps and clears the
    counts, and later launches run normally."""
    from mcgb import _lib
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    b = LadderBatch(XYModel(), [(16, np.geomspace(0.8, 1.2, 4))], exchange_interval=2, proposal="gaussian",
                    cluster_size=2, threads=128)
    assert b.resident
    b.run(20)
    b.check_errors()
    old = b.set_wait_limit(0)
    try:
        b.run(20)
        with pytest.raises(_lib.MCGBTimeout):
            b.check_errors()
    finally:
        b.set_wait_limit(None)
    assert old == b.set_wait_limit(None)
    w2t, t2w = b.w2t.copy_to_host(), b.t2w.copy_to_host()
    np.testing.assert_array_equal(t2w[w2t], np.arange(4))
    np.testing.assert_array_equal(b.betas.copy_to_host(), b._initial_betas[w2t])
    assert not b.sync.copy_to_host().any()
    b.run(20)
    b.check_errors()
    w2t, t2w = b.w2t.copy_to_host(), b.t2w.copy_to_host()
    np.testing.assert_array_equal(t2w[w2t], np.arange(4))
    np.testing.assert_array_equal(b.betas.copy_to_host(), b._initial_betas[w2t])


def test_autotune_with_samples_leaves_the_chain_and_the_ring_alone():
    """Autotuning with a sample cadence times its trials with a scratch ring,
    then restores the caller's ring and the chain: the run afterwards equals
    an untuned twin's on the same shape, samples included."""
    from mcgb.batch import LadderBatch
    from mcgb.models.ising.model import IsingModel
    init = seeded_spins(np.random.default_rng(12), 4, 32)
    kw = dict(seeds=[21], exchange_interval=5, initial_states=[init])
    a = LadderBatch(IsingModel(), [(32, np.geomspace(2.0, 2.6, 4))], **kw)
    b = LadderBatch(IsingModel(), [(32, np.geomspace(2.0, 2.6, 4))], **kw)
    for x in (a, b):
        x.allocate_samples(5, 5, 8)
        x.run(10)
    before = a.samples.copy_to_host()
    ring = (a.n_slots, a.first_sample_sweep, a.sample_interval)
    trials = a.autotune(sample_interval=1, shapes=[(1, 128), (2, 128), (4, 64)])
    assert len(trials) == 3 and (a.cluster_size, a.threads) in [(C, T) for _, C, T in trials]
    assert (a.n_slots, a.first_sample_sweep, a.sample_interval) == ring
    np.testing.assert_array_equal(a.samples.copy_to_host(), before)
    b.configure(a.cluster_size, a.threads)
    for x in (a, b):
        x.run(20)
        x.check_errors()
    np.testing.assert_array_equal(a.ladder_state(0), b.ladder_state(0))
    for name in ("samples", "w2t", "energies", "clock"):
        np.testing.assert_array_equal(getattr(a, name).copy_to_host(), getattr(b, name).copy_to_host(), err_msg=name)


def test_autotune_of_a_ragged_batch_times_real_steps_and_puts_everything_back():
    """Choosing between one launch and one launch per size runs a few real
    steps of each (exchanges, resident launches, graphs); afterwards the chain
    continues exactly as an untuned twin's with the grouping and shapes
    autotune chose: states, maps, counters, round trips, samples, clock."""
    from mcgb.batch import LadderBatch
    from mcgb.models.ising.model import IsingModel
    rng = np.random.default_rng(31)
    ladders = [(16, list(np.geomspace(2.0, 2.6, 6))), (32, list(np.geomspace(2.0, 2.6, 5)))]
    inits = [seeded_spins(rng, len(T), L) for L, T in ladders]
    kw = dict(seeds=[8, 9], exchange_interval=5, initial_states=inits)
    a = LadderBatch(IsingModel(), ladders, **kw)
    b = LadderBatch(IsingModel(), ladders, **kw)
    for x in (a, b):
        x.allocate_samples(5, 5, 16)
        x.run(10)
    a.autotune(sample_interval=5, shapes=[(1, 128), (2, 128)])
    if len(a.groups) > 1:
        b.split_by_size(True)
    for ga, gb in zip(a.groups, b.groups):
        b._configure_group(gb, ga.cluster_size, ga.threads)
    b._graphs.clear()
    assert [list(ga.idx) for ga in a.groups] == [list(gb.idx) for gb in b.groups]
    for x in (a, b):
        x.run(30)
        x.check_errors()
    for k in range(2):
        np.testing.assert_array_equal(a.ladder_state(k), b.ladder_state(k))
    for name in ("w2t", "t2w", "betas", "swap_counts", "trips", "energies", "clock", "samples"):
        np.testing.assert_array_equal(getattr(a, name).copy_to_host(), getattr(b, name).copy_to_host(), err_msg=name)
    assert a.sweeps == b.sweeps == 40 and a.exchange_rounds == b.exchange_rounds == 8


def test_bulk_strip_loads_equal_per_thread_loads():
    """XY ladder of 128^2 replicas in the shared-memory stream variant (4 CTAs
    x 1024 threads): fused window + exchange launches, whose strips, angles
    and streams arrive by bulk copies, against the window-only launches
    with per-thread loads followed by the separate exchange kernel (the
    warm-up path): identical chains, streams, maps, counters and energies."""
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    temps = np.geomspace(0.7, 1.2, 4)
    init = np.random.default_rng(31).uniform(-np.pi, np.pi, (4, 128, 128)).astype(np.float32)
    kw = dict(seeds=[9], exchange_interval=5, cluster_size=4, threads=1024, initial_states=[init], resident=False)
    a, b = LadderBatch(XYModel(), [(128, temps)], **kw), LadderBatch(XYModel(), [(128, temps)], **kw)
    a.run(40, graph=False)
    b.run(40, tune=True, graph=False)
    a.check_errors()
    np.testing.assert_array_equal(a.ladder_state(0), b.ladder_state(0))
    for name in ("rng", "aux", "w2t", "t2w", "betas", "swap_counts", "trips", "e_run", "energies", "accepted",
                 "clock"):
        np.testing.assert_array_equal(getattr(a, name).copy_to_host(), getattr(b, name).copy_to_host(),
                                      err_msg=name)
