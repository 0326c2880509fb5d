"""Fixtures produced by the reference's own kernels and host classes.

    python tests/golden/make_reference_kernel_golden.py --reference <checkout>
    (or set MCGB_REFERENCE to the checkout)

Numba is absent here, so the reference's modules run UNMODIFIED on the CPU
under the pure-Python ``numba`` stand-in in ``numba_standin/`` (its
docstring says what it emulates and where it differs from compiled code).
The script drives the reference exactly as its users do --
``Runtime(model, L, T, seed)``, ``ParallelTempering(runtime, ...)``,
``Simulation(pt, ...).run()``, ``He3GaussianRuntime`` -- after writing a
seeded initial state with ``state.copy_to_device``, and stores every input
and output in ``reference_kernels.npz``:

* ``<case>/in``: the injected state; ``<case>/betas``, ``seed``, ...;
* ``<case>/out``: the final state in walker order, ``<case>/rng_out``: every
  per-site stream after the run;
* ``<case>/measure/<channel>``: ``Runtime.measure()`` of the final state
  (and ``measure_t/<channel>`` with a temperature order), ``<case>/energy``:
  ``measure_energy``;
* for ParallelTempering + Simulation cases: ``samples/<channel>``, the
  metadata (``sample_sweeps``), the PT diagnostics (attempts, accepted,
  maps, round trips, walker history) and the exchange streams.

The Ising cases use the temperatures 1.5, 2.269 and 3.0 only, whose CUDA
``expf`` values ``ising_cuda_expf.json`` holds: with that table installed
the stand-in's acceptance test sees exactly the GPU's float32 exponentials,
and the script checks that no other Ising argument was evaluated.
"""

import argparse
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "reference_kernels.npz"
ISING_T = [1.5, 2.269, 3.0]


def load_expf_table():
    cap = json.loads((HERE / "ising_cuda_expf.json").read_text())
    table = {}
    for args, vals in zip(cap["arguments_f32_bits"], cap["expf_f32_bits"]):
        for a, v in zip(args, vals):
            table[int(a, 16)] = int(v, 16)
    return table


def seeded_state(kind, R, L, seed):
    r = np.random.default_rng(seed)
    if kind == "ising":
        return r.choice(np.array([-1, 1], np.int8), (R, L, L))
    if kind == "xy":
        # Uniform in [0, 2 pi), wrapped to [-pi, pi) as the kernel assumes.
        t = r.uniform(0, 2 * np.pi, (R, L, L)).astype(np.float32)
        return np.where(t >= np.float32(np.pi), t - np.float32(2 * np.pi), t).astype(np.float32)
    if kind == "kawamura":
        s = np.zeros((R, L, L, 5), np.float32)
        s[..., 0] = r.uniform(-np.pi, np.pi, (R, L, L))
        s[..., 1] = r.choice([-1.0, 1.0], (R, L, L))
        d = r.normal(size=(R, L, L, 3))
        s[..., 2:] = d / np.linalg.norm(d, axis=-1, keepdims=True)
        return s
    if kind == "he3":
        a = 0.3 * np.sqrt(2)
        re = r.uniform(-a, a, (R, L, L, 3, 2))
        im = r.uniform(-a, a, (R, L, L, 3, 2))
        return (re + 1j * im).astype(np.complex64)
    raise ValueError(kind)


def put(dest, prefix, **items):
    for k, v in items.items():
        dest[f"{prefix}/{k}"] = np.asarray(v)


def put_params(dest, prefix, model, **extra):
    """The model's float32 parameters as the kernels receive them."""
    for k in ("J", "delta", "K", "g_d"):
        if hasattr(model, k):
            dest[f"{prefix}/params/{k}"] = np.asarray(getattr(model, k), np.float32)
    if hasattr(model, "betas"):
        dest[f"{prefix}/params/coefficients"] = np.asarray(model.betas, np.float32)
    if getattr(model, "pressure", None) is not None:
        dest[f"{prefix}/params/pressure"] = np.asarray(model.pressure, np.float64)
        dest[f"{prefix}/params/reduced_temperature"] = np.asarray(model.reduced_temperature, np.float64)
    for k, v in extra.items():
        dest[f"{prefix}/params/{k}"] = np.asarray(v, np.float32)
    dest[f"{prefix}/parameters_repr"] = np.asarray(repr(model.parameters()))


def put_measure(out, prefix, name, m):
    for ch, v in m.items():
        out[f"{prefix}/{name}/{ch}"] = np.asarray(v)


def runtime_case(out, name, kind, model, L, T, seed, sweeps, cls=None, **kw):
    from core.runtime import Runtime
    cls = cls or Runtime
    rt = cls(model, L, T, seed=seed, **kw)
    state = seeded_state(kind, rt.R, L, seed + 1000)
    rt.state.copy_to_device(state)
    for _ in range(sweeps):
        rt.sweep()
    from numba import cuda
    energy = cuda.device_array(rt.R, np.float64)
    rt.measure_energy(energy)
    order = np.arange(rt.R, dtype=np.int32)[::-1].copy()
    put(out, name, kind=kind, L=L, T=np.asarray(T, np.float64), seed=seed, sweeps=sweeps,
        betas=rt.betas.copy_to_host(), **{"in": state}, out=rt.snapshot(),
        rng_out=rt.rng_states.copy_to_host(), energy=energy.copy_to_host(), measure_order=order)
    put_params(out, name, model, **{k: v for k, v in kw.items() if k in ("rho", "proposal_mass")})
    put_measure(out, name, "measure", rt.measure())
    put_measure(out, name, "measure_t", rt.measure(temperature_indices=cuda.to_device(order)))
    return rt


def pt_sim_case(out, name, kind, model, L, T, seed, interval, therm, meas, every, tracked, stride):
    from core.parallel_tempering import ParallelTempering
    from core.runtime import Runtime
    from core.simulation import Simulation
    rt = Runtime(model, L, T, seed=seed)
    state = seeded_state(kind, rt.R, L, seed + 1000)
    rt.state.copy_to_device(state)
    pt = ParallelTempering(rt, exchange_interval=interval, tracked_walkers=tracked, history_stride=stride)
    res = Simulation(pt, thermalization_sweeps=therm, measurement_sweeps=meas, sample_interval=every).run()
    meta = res["metadata"]
    diag = meta["parallel_tempering"]
    put(out, name, kind=kind, L=L, T=np.asarray(T, np.float64), seed=seed, interval=interval,
        thermalization=therm, measurement=meas, sample_interval=every, tracked=np.asarray(tracked),
        history_stride=stride, **{"in": state}, out=rt.snapshot(), out_t=pt.snapshot(),
        rng_out=rt.rng_states.copy_to_host(), exchange_rng_out=pt._rng_states.copy_to_host(),
        betas_out=rt.betas.copy_to_host(), energies=pt.energies.copy_to_host(),
        sample_sweeps=meta["sample_sweeps"])
    for k in ("exchange_seed", "sweeps", "exchange_rounds", "next_parity", "temperature_betas", "attempts",
              "accepted", "acceptance_rates", "walker_to_temperature", "temperature_to_walker",
              "walker_round_trips", "walker_round_trip_total_sweeps"):
        out[f"{name}/pt/{k}"] = np.asarray(diag[k])
    out[f"{name}/pt/mean_round_trip_sweeps"] = np.asarray(
        np.nan if diag["mean_round_trip_sweeps"] is None else diag["mean_round_trip_sweeps"])
    hist = diag["walker_history"]
    for k in ("walker_ids", "sweeps", "exchange_rounds", "temperature_indices"):
        out[f"{name}/pt/history/{k}"] = np.asarray(hist[k])
    put_params(out, name, model)
    put_measure(out, name, "samples", res["samples"])


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
    sys.path.insert(0, str(HERE / "numba_standin"))
    from numba import cuda
    from models.he3.model import He3Model
    from models.he3.sampling import He3GaussianRuntime
    from models.ising.model import IsingModel
    from models.kawamura.model import KawamuraModel
    from models.xy.model import XYModel

    cuda.set_expf_table(load_expf_table())
    out = {}
    cuda.clear_expf_misses()
    runtime_case(out, "ising_rt", "ising", IsingModel(J=1.0), 16, ISING_T, 58, 20)
    pt_sim_case(out, "ising_pt", "ising", IsingModel(J=1.0), 8, ISING_T, 50, interval=2, therm=6, meas=12,
                every=3, tracked=[0, 2], stride=2)
    if cuda.expf_misses():
        raise AssertionError(f"Ising exponentials without a CUDA value: {sorted(cuda.expf_misses())}")

    runtime_case(out, "xy_rt", "xy", XYModel(J=1.0, delta=1.5), 16, [0.8, 1.1], 60, 6)
    pt_sim_case(out, "xy_pt", "xy", XYModel(J=1.0, delta=1.5), 8, list(np.geomspace(0.7, 1.2, 4)), 61,
                interval=2, therm=4, meas=8, every=2, tracked=[0, 1, 2, 3], stride=1)
    runtime_case(out, "kawamura_rt", "kawamura", KawamuraModel(J=1.0, delta=1.5), 8, [0.65, 0.8], 62, 4)
    pt_sim_case(out, "kawamura_pt", "kawamura", KawamuraModel(J=1.0, delta=1.5), 8,
                list(np.linspace(0.65, 0.80, 3)), 63, interval=2, therm=2, meas=4, every=2, tracked=[1],
                stride=1)
    runtime_case(out, "he3_rt", "he3", He3Model(), 8, [0.35, 0.45], 64, 3)
    runtime_case(out, "he3p_rt", "he3", He3Model(pressure=20, g_d=0.001), 6, [0.35, 0.45], 65, 3)
    rt = runtime_case(out, "he3g_rt", "he3", He3Model(), 8, [0.35, 0.45], 66, 3, cls=He3GaussianRuntime,
                      rho=-0.9, proposal_mass=0.0)
    diag = rt.sampling_diagnostics()
    for k in ("attempts", "accepted", "nonfinite_rejections"):
        out[f"he3g_rt/diag/{k}"] = np.asarray(diag[k], np.int64)
    out["he3g_rt/counts"] = rt.gaussian.counts.copy_to_host()
    pt_sim_case(out, "he3_pt", "he3", He3Model(), 6, [0.33, 0.40, 0.47], 67, interval=1, therm=1, meas=2,
                every=1, tracked=[0, 2], stride=1)

    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT.name}: {len(out)} arrays, {OUT.stat().st_size} bytes")


if __name__ == "__main__":
    main()
