"""Golden vectors produced by the reference's own Python code.

    python tests/golden/make_reference_golden.py --reference <checkout>
    (or set MCGB_REFERENCE to the checkout)

The reference's run-file writer (utils/data_io.py) and temperature-ladder
builder (utils/temperature_ladder.py) import only numpy and json, so they run
here as they are.  This script imports them from the checkout and writes

* ``temperature_ladders.json`` -- make_temperature_ladder's output (float64
  bit patterns) for uniform-beta and focused ladders of the reference's
  studies, and the error message of each invalid request;
* ``runs_v1_reference.npz`` -- a two-size run file written by its save_runs
  (samples and PT diagnostics metadata), which ``mcgb.runs.load_runs`` must
  read back exactly.
"""

import argparse
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

LADDERS = [
    {"T_min": 0.70, "T_max": 1.20, "n_T": 32},
    {"T_min": 0.33, "T_max": 0.47, "n_T": 24},
    {"T_min": 2.0, "T_max": 2.5, "n_T": 64, "Tc": 2.269},
    {"T_min": 0.78, "T_max": 1.02, "n_T": 64, "Tc": 0.893},
    {"T_min": 0.65, "T_max": 0.80, "n_T": 48, "Tc": 0.72, "tc_window": 0.04, "tc_fraction": 0.3},
    {"T_min": 1.0, "T_max": 3.0, "n_T": 7, "Tc": 2.0, "tc_window": 0.5, "tc_fraction": 0.75},
]
INVALID = [
    {"T_min": 1.2, "T_max": 0.7, "n_T": 8},
    {"T_min": 0.7, "T_max": 1.2, "n_T": 1},
    {"T_min": 0.7, "T_max": 1.2, "n_T": 8, "Tc": 1.19},
    {"T_min": 0.7, "T_max": 1.2, "n_T": 8, "Tc": 0.9, "tc_fraction": 1.0},
    {"T_min": 0.7, "T_max": 1.2, "n_T": 8, "Tc": 0.9, "tc_window": 0.01, "tc_fraction": 0.99},
]


def sample_runs():
    r = np.random.default_rng(5)
    runs = {}
    for L, R in ((8, 4), (16, 3)):
        T = np.geomspace(0.8, 1.2, R)
        samples = {"energy": r.normal(size=(50, R)), "mx": r.normal(size=(50, R)),
                   "twist_sin_x": r.normal(size=(50, R))}
        meta = {"L": L, "temperatures": T, "seed": 42 + L, "model_parameters": {"J": np.float32(1.37)},
                "thermalization_sweeps": 100, "measurement_sweeps": 500, "sample_interval": 10,
                "sample_sweeps": 100 + 10 * np.arange(1, 51),
                "parallel_tempering": {"exchange_interval": 10, "exchange_seed": 43 + L, "sweeps": 600,
                                       "exchange_rounds": 60, "next_parity": 0,
                                       "diagnostics_scope": "since_wrapper_creation_including_thermalization",
                                       "attempts": np.full(R - 1, 30), "accepted": np.arange(R - 1) + 7,
                                       "acceptance_rates": (np.arange(R - 1) + 7) / 30,
                                       "walker_to_temperature": np.arange(R)[::-1].copy(),
                                       "temperature_to_walker": np.arange(R)[::-1].copy(),
                                       "walker_round_trips": np.arange(R), "walker_round_trip_total_sweeps":
                                       np.arange(R) * 100, "mean_round_trip_sweeps": None}}
        runs[L] = {"samples": samples, "metadata": meta}
    return runs


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--reference", default=os.environ.get("MCGB_REFERENCE"),
                    help="path of the reference checkout (or MCGB_REFERENCE)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("give --reference or set MCGB_REFERENCE")
    # The checkout is read-only: import it without writing bytecode there.
    sys.dont_write_bytecode = True
    sys.path.insert(0, str(Path(args.reference).resolve()))
    from utils.data_io import save_runs
    from utils.temperature_ladder import make_temperature_ladder

    cases = []
    for kw in LADDERS:
        T = make_temperature_ladder(**kw)
        cases.append({"args": kw, "temperatures_f64_hex": [float(t).hex() for t in T]})
    errors = []
    for kw in INVALID:
        try:
            make_temperature_ladder(**kw)
        except ValueError as e:
            errors.append({"args": kw, "error": str(e)})
        else:
            raise AssertionError(f"expected an error for {kw}")
    (HERE / "temperature_ladders.json").write_text(json.dumps({"ladders": cases, "invalid": errors}, indent=1) + "\n")
    save_runs(HERE / "runs_v1_reference.npz", sample_runs())
    print("wrote temperature_ladders.json and runs_v1_reference.npz")


if __name__ == "__main__":
    main()
