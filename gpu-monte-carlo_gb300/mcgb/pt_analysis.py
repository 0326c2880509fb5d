"""Summaries of parallel-tempering diagnostics saved with each run.

``pt_summary`` computes, for every run whose metadata carries the
``parallel_tempering`` diagnostics dictionary (``ParallelTempering.diagnostics``
or ``LadderBatch.diagnostics``), the numbers of utils/Analysis/parallel_tempering.py:7-50
``PTAnalysis.summary``: per-pair and aggregate swap acceptance, completed
round trips per walker and their mean duration, the counter scope and
whether a walker history was recorded (which is validated as there).
``format_summary`` is the text report.  Plotting is left to the caller.

The counters themselves are kept on the GPU by the exchange kernels (swap
attempts/acceptances per pair, round-trip bookkeeping per walker), so a
summary needs only the small diagnostic arrays copied once per run.
"""

import numpy as np


def _validate_history(L, history, n_temps):
    ids = np.asarray(history["walker_ids"], dtype=np.int64)
    sweeps = np.asarray(history["sweeps"], dtype=np.int64)
    pos = np.asarray(history["temperature_indices"])
    if (ids.ndim != 1 or len(ids) == 0 or len(np.unique(ids)) != len(ids) or np.any(ids < 0)
            or np.any(ids >= n_temps) or sweeps.ndim != 1 or len(sweeps) == 0 or np.any(np.diff(sweeps) < 0)
            or pos.shape != (len(sweeps), len(ids)) or not np.issubdtype(pos.dtype, np.integer)
            or np.any(pos < 0) or np.any(pos >= n_temps)):
        raise ValueError(f"L={L}: invalid walker history")


def pt_summary(runs):
    """``{L: summary}`` for the runs of ``{L: run}`` that used parallel tempering."""
    out = {}
    for L, run in sorted(runs.items()):
        meta = run["metadata"]
        if "parallel_tempering" not in meta:
            continue
        pt = meta["parallel_tempering"]
        attempts = np.asarray(pt["attempts"])
        accepted = np.asarray(pt["accepted"])
        trips = np.asarray(pt["walker_round_trips"])
        trip_sweeps = np.asarray(pt["walker_round_trip_total_sweeps"])
        T = np.asarray(meta["temperatures"], dtype=float)
        history = pt.get("walker_history")
        if history is not None:
            _validate_history(L, history, len(T))
        out[L] = {
            "temperatures": T.tolist(),
            "attempts": attempts.tolist(),
            "accepted": accepted.tolist(),
            "acceptance_rates": [float(a / n) if n else None for a, n in zip(accepted, attempts)],
            "aggregate_acceptance": float(accepted.sum() / attempts.sum()) if attempts.sum() else None,
            "walker_round_trips": trips.tolist(),
            "walker_mean_round_trip_sweeps": [float(t / n) if n else None for t, n in zip(trip_sweeps, trips)],
            "mean_round_trip_sweeps": float(trip_sweeps.sum() / trips.sum()) if trips.sum() else None,
            "diagnostics_scope": pt["diagnostics_scope"],
            "history_available": history is not None,
        }
    return out


def format_summary(summary):
    lines = ["Parallel tempering diagnostics (including thermalization)",
             "Trip means exclude unfinished trips; zero trips does not imply zero one-way crossings."]
    for L, s in summary.items():
        lines.append(f"L={L}: {sum(s['accepted'])}/{sum(s['attempts'])} accepted, "
                     f"{sum(s['walker_round_trips'])} trips, mean {s['mean_round_trip_sweeps']} sweeps/trip")
        lines.append("  walker paths recorded" if s["history_available"]
                     else "  walker paths were not recorded; final mappings cannot reconstruct trajectories")
    return "\n".join(lines)
