"""Run files, temperature ladders and PT summaries (CPU).

Golden vectors come from the reference's own code (tests/golden/
make_reference_golden.py): its temperature ladders, and a run file written by
its save_runs.  The PT-summary cases port tests/test_pt_analysis.py:15-66.
"""

import copy
import json
import sys
import zipfile
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "gpu-monte-carlo_gb300"))

from mcgb import ladder, pt_analysis, runs  # noqa: E402


# ------------------------------------------------------------ ladders

def ladder_cases():
    return json.loads((GOLDEN / "temperature_ladders.json").read_text())


@pytest.mark.parametrize("case", ladder_cases()["ladders"], ids=lambda c: json.dumps(c["args"]))
def test_ladders_match_the_reference(case):
    want = np.array([float.fromhex(h) for h in case["temperatures_f64_hex"]])
    got = ladder.make_temperature_ladder(**case["args"])
    np.testing.assert_allclose(got, want, rtol=1e-13, atol=0)
    assert np.all(np.diff(got) > 0)
    assert got[0] == pytest.approx(case["args"]["T_min"]) and got[-1] == pytest.approx(case["args"]["T_max"])


@pytest.mark.parametrize("case", ladder_cases()["invalid"], ids=lambda c: json.dumps(c["args"]))
def test_invalid_ladders_raise_the_reference_errors(case):
    with pytest.raises(ValueError, match=case["error"]):
        ladder.make_temperature_ladder(**case["args"])


def test_focused_ladder_puts_the_requested_fraction_in_the_window():
    T = ladder.make_temperature_ladder(2.0, 2.5, 201, Tc=2.269, tc_window=0.08, tc_fraction=0.6)
    inside = np.mean((T > 2.269 - 0.04) & (T < 2.269 + 0.04))
    assert inside == pytest.approx(0.6, abs=0.02)


def test_ragged_ladders_repeat_the_ladder_per_size():
    out = ladder.ragged_ladders([16, 32], 0.78, 1.02, 8, ladders_per_size=2, Tc=0.893)
    assert [L for L, _ in out] == [16, 16, 32, 32]
    for _, T in out:
        np.testing.assert_array_equal(T, out[0][1])


def test_adapt_ladder_equalises_acceptance_and_keeps_the_ends():
    T = np.geomspace(0.7, 1.2, 6)
    rates = [0.1, 0.5, 0.5, 0.5, 0.9]
    new = ladder.adapt_ladder(T, rates)
    assert new[0] == pytest.approx(T[0]) and new[-1] == pytest.approx(T[-1])
    assert np.all(np.diff(new) > 0)
    b, nb = 1 / T[::-1], 1 / new[::-1]
    # Rates are in temperature order: the hard pair (0.1) is the coldest,
    # the last gap in beta order, and shrinks; the easy hot pair (0.9) grows.
    assert np.diff(nb)[-1] < np.diff(b)[-1] and np.diff(nb)[0] > np.diff(b)[0]
    np.testing.assert_array_equal(ladder.adapt_ladder(T, [None] * 5), T)
    with pytest.raises(ValueError):
        ladder.adapt_ladder(T, rates[:3])


# ------------------------------------------------------------ run files

def test_reference_run_file_loads_exactly():
    loaded = runs.load_runs(GOLDEN / "runs_v1_reference.npz")
    assert sorted(loaded) == [8, 16]
    with np.load(GOLDEN / "runs_v1_reference.npz") as f:
        manifest = json.loads(f["manifest"].item())
        for L, run in loaded.items():
            assert list(run["samples"]) == manifest["runs"][str(L)]["sample_names"]
            for name, values in run["samples"].items():
                np.testing.assert_array_equal(values, f[f"L{L}_{name}"])
            assert run["metadata"] == manifest["runs"][str(L)]["metadata"]
    assert loaded[8]["metadata"]["parallel_tempering"]["attempts"] == [30, 30, 30]


def test_saved_file_has_the_reference_layout_and_round_trips(tmp_path):
    ref = runs.load_runs(GOLDEN / "runs_v1_reference.npz")
    path = tmp_path / "out" / "pt_run.npz"
    runs.save_runs(path, ref)
    with zipfile.ZipFile(path) as z:
        names = sorted(z.namelist())
    with zipfile.ZipFile(GOLDEN / "runs_v1_reference.npz") as z:
        assert names == sorted(z.namelist())
    with np.load(path) as mine, np.load(GOLDEN / "runs_v1_reference.npz") as theirs:
        assert json.loads(mine["manifest"].item()) == json.loads(theirs["manifest"].item())
        for key in theirs.files:
            if key != "manifest":
                np.testing.assert_array_equal(mine[key], theirs[key])
                assert mine[key].dtype == theirs[key].dtype
    assert not [p for p in path.parent.iterdir() if p.name.endswith(".tmp")]


def test_numpy_metadata_is_saved_as_json_values(tmp_path):
    """tests/test_parallel_tempering.py:277-286: samples and PT diagnostics
    survive a save/load round trip."""
    diag = {"attempts": np.array([3, 4]), "accepted": np.array([1, 2]), "acceptance_rates": np.array([1 / 3, 0.5]),
            "mean_round_trip_sweeps": None, "exchange_seed": np.int64(7), "scale": np.float32(0.5)}
    run = {"samples": {"energy": np.arange(6.0).reshape(3, 2), "magnetization": np.ones((3, 2))},
           "metadata": {"L": 4, "temperatures": np.array([1.0, 2.0]), "parallel_tempering": diag}}
    runs.save_runs(tmp_path / "r.npz", {4: run})
    back = runs.load_runs(tmp_path / "r.npz")[4]
    for name, values in run["samples"].items():
        np.testing.assert_array_equal(back["samples"][name], values)
    for name, value in diag.items():
        np.testing.assert_equal(back["metadata"]["parallel_tempering"][name], value)


def test_unknown_versions_are_rejected(tmp_path):
    np.savez_compressed(tmp_path / "v2.npz", manifest=np.array(json.dumps({"version": 2, "runs": {}})))
    with pytest.raises(ValueError, match="Unsupported data format version"):
        runs.load_runs(tmp_path / "v2.npz")


def test_runs_by_size_refuses_duplicate_sizes():
    a = {"samples": {}, "metadata": {"L": 8}}
    assert list(runs.runs_by_size([a, {"samples": {}, "metadata": {"L": 16}}])) == [8, 16]
    with pytest.raises(ValueError):
        runs.runs_by_size([a, copy.deepcopy(a)])


# ------------------------------------------------------------ PT summaries

def saved_run():
    return {"samples": {}, "metadata": {
        "L": 16, "temperatures": [0.8, 0.9, 1.0],
        "parallel_tempering": {
            "exchange_interval": 10, "exchange_seed": 9, "sweeps": 1000, "exchange_rounds": 100,
            "next_parity": 0, "diagnostics_scope": "since_wrapper_creation_including_thermalization",
            "attempts": [50, 50], "accepted": [40, 10], "acceptance_rates": [0.8, 0.2],
            "walker_to_temperature": [2, 0, 1], "temperature_to_walker": [1, 2, 0],
            "walker_round_trips": [2, 1, 0], "walker_round_trip_total_sweeps": [600, 400, 0],
            "mean_round_trip_sweeps": 1000 / 3}}}


def test_weighted_rates_and_completed_trip_times():
    run = saved_run()
    run["metadata"]["parallel_tempering"].update(attempts=[50, 25], accepted=[40, 10])
    s = pt_analysis.pt_summary({16: run})[16]
    assert s["aggregate_acceptance"] == 50 / 75
    assert s["acceptance_rates"] == [0.8, 0.4]
    assert s["walker_round_trips"] == [2, 1, 0]
    assert s["walker_mean_round_trip_sweeps"] == [300, 400, None]
    assert s["mean_round_trip_sweeps"] == pytest.approx(1000 / 3)
    assert s["diagnostics_scope"] == "since_wrapper_creation_including_thermalization"
    json.dumps(s, allow_nan=False)


def test_unattempted_edges_and_unfinished_trips_have_no_mean():
    run = saved_run()
    run["metadata"]["parallel_tempering"].update(attempts=[0, 0], accepted=[0, 0], walker_round_trips=[0, 0, 0],
                                                 walker_round_trip_total_sweeps=[0, 0, 0])
    s = pt_analysis.pt_summary({16: run})[16]
    assert s["acceptance_rates"] == [None, None]
    assert s["aggregate_acceptance"] is None and s["mean_round_trip_sweeps"] is None


def test_ordinary_runs_are_skipped():
    assert list(pt_analysis.pt_summary({16: saved_run(), 32: {"metadata": {}}})) == [16]
    assert pt_analysis.pt_summary({32: {"metadata": {}}}) == {}
    text = pt_analysis.format_summary(pt_analysis.pt_summary({16: saved_run()}))
    assert "L=16: 50/100 accepted, 3 trips" in text and "not recorded" in text


def test_invalid_history_is_rejected():
    run = saved_run()
    run["metadata"]["parallel_tempering"]["walker_history"] = {
        "walker_ids": [0, 0], "sweeps": [10, 20], "temperature_indices": [[0, 1], [1, 2]]}
    with pytest.raises(ValueError, match="invalid walker history"):
        pt_analysis.pt_summary({16: run})
    run["metadata"]["parallel_tempering"]["walker_history"] = {
        "walker_ids": [0, 2], "sweeps": [10, 20], "temperature_indices": [[0, 1], [1, 2]]}
    assert pt_analysis.pt_summary({16: run})[16]["history_available"]


def test_work_lists_cost_visits_per_thread():
    """Work lists weigh a replica by the visits each thread makes per colour
    phase, so a lattice smaller than the block is not taken for nearly free:
    on 4 x 256, L=32 (64 plaquettes a CTA) costs one visit, L=128 four."""
    from mcgb.batch import lpt_work_lists, visit_costs
    Ls = np.repeat([32, 128], 4)
    costs = visit_costs(Ls, 4, 256)
    assert list(costs) == [1.5] * 4 + [4.5] * 4
    wp, wi, loads = lpt_work_lists(costs, 4)
    for k in range(4):
        assert sorted(Ls[wi[wp[k]:wp[k + 1]]]) == [32, 128]
    np.testing.assert_allclose(loads, 6.0)
