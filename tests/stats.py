"""Block-jackknife estimators for the statistical parity tests.

The estimators are the reference's analysis formulas for each model
(models/ising/analysis.py:55-75, models/xy/analysis.py:29-55,
models/kawamura/analysis.py:36-53, models/he3/analysis.py:29-41); errors come
from a delete-one-block jackknife over time blocks, the procedure of
utils/Analysis/statistics.py:5-37.  Inputs are ``{"samples": {channel: (n, T)}}``
run dictionaries as ``Simulation.run`` returns them.
"""

import math

import numpy as np


def blocks_of(x, block_size):
    """Means of consecutive complete time blocks of ``x`` (n, ...) -> (B, ...)."""
    x = np.asarray(x, dtype=np.float64)
    B = len(x) // block_size
    if B < 2:
        raise ValueError("need at least two complete time blocks")
    return x[:B * block_size].reshape((B, block_size) + x.shape[1:]).mean(axis=1)


def jackknife(moments, estimator, block_size):
    """Estimate and jackknife error of ``estimator(mean_moments)``."""
    blocks = {k: blocks_of(v, block_size) for k, v in moments.items()}
    B = len(next(iter(blocks.values())))
    total = {k: v.sum(axis=0) for k, v in blocks.items()}
    value = estimator({k: t / B for k, t in total.items()})
    leave_one_out = np.stack([estimator({k: (total[k] - blocks[k][b]) / (B - 1) for k in blocks})
                              for b in range(B)])
    spread = leave_one_out - leave_one_out.mean(axis=0)
    error = np.sqrt((B - 1) / B * (spread ** 2).sum(axis=0))
    return value, error


def xy_observables(samples, L, temperatures, J=1.0, block_size=100):
    """Energy per site, Binder cumulant 1 - <m^4>/(2<m^2>^2), helicity
    modulus (models/xy/analysis.py:47-54) and <|m|> per site."""
    T = np.asarray(temperatures, dtype=np.float64)
    m2 = np.asarray(samples["mx"]) ** 2 + np.asarray(samples["my"]) ** 2
    qx = np.asarray(samples["twist_sin_x"], dtype=np.float64)
    moments = {"e": np.asarray(samples["energy"]) / L ** 2, "m2": m2, "m4": m2 ** 2,
               "cx": np.asarray(samples["twist_cos_x"]), "qx": qx, "qx2": qx ** 2,
               "absm": np.sqrt(m2) / L ** 2}

    def est(m):
        helicity = (J * m["cx"] - J ** 2 / T * (m["qx2"] - m["qx"] ** 2)) / L ** 2
        return np.stack((m["e"], 1 - m["m4"] / (2 * m["m2"] ** 2), helicity, m["absm"]))

    value, error = jackknife(moments, est, block_size)
    return dict(zip(("energy", "binder", "helicity", "magnetization"), zip(value, error)))


def linear_crossings(T, y1, y2):
    """Temperatures where two piecewise-linear curves cross (the method of
    utils/Analysis/crossings.py:5-24): sample points where they agree and
    linear interpolation inside every sign change of y1 - y2."""
    T = np.asarray(T, dtype=np.float64)
    d = np.asarray(y1, dtype=np.float64) - np.asarray(y2, dtype=np.float64)
    if not np.all(np.isfinite(d)) or np.any((d[:-1] == 0) & (d[1:] == 0)):
        return []
    roots = list(T[d == 0])
    for i in np.where(d[:-1] * d[1:] < 0)[0]:
        roots.append(T[i] - d[i] * (T[i + 1] - T[i]) / (d[i + 1] - d[i]))
    return sorted(float(t) for t in roots)


def binder_crossing(samples_a, samples_b, temperatures, binder, block_size):
    """The unique crossing of two sizes' Binder curves with its block
    jackknife error, or None when the full-sample curves do not cross once
    (``binder(moments) -> curve`` maps block means of the "m2", "m4" moments
    to the Binder curve)."""
    def moments(samples):
        m2 = np.asarray(samples["m2"], np.float64)
        return {"m2": m2, "m4": m2 ** 2}
    ma, mb = moments(samples_a), moments(samples_b)
    ba = {k: blocks_of(v, block_size) for k, v in ma.items()}
    bb = {k: blocks_of(v, block_size) for k, v in mb.items()}
    B = min(len(ba["m2"]), len(bb["m2"]))
    ta = {k: v[:B].sum(0) for k, v in ba.items()}
    tb = {k: v[:B].sum(0) for k, v in bb.items()}
    full = linear_crossings(temperatures, binder({k: v / B for k, v in ta.items()}),
                            binder({k: v / B for k, v in tb.items()}))
    if len(full) != 1:
        return None
    est = []
    for b in range(B):
        c = linear_crossings(temperatures, binder({k: (ta[k] - ba[k][b]) / (B - 1) for k in ta}),
                             binder({k: (tb[k] - bb[k][b]) / (B - 1) for k in tb}))
        est.append(c[0] if len(c) == 1 else np.nan)
    est = np.asarray(est)
    if not np.all(np.isfinite(est)):
        return None
    return full[0], float(np.sqrt((B - 1) / B * ((est - est.mean()) ** 2).sum()))


def energy_observable(samples, L, block_size=100):
    value, error = jackknife({"e": np.asarray(samples["energy"]) / L ** 2}, lambda m: m["e"][None], block_size)
    return {"energy": (value[0], error[0])}


def ising_observables(samples, L, temperatures, block_size=100):
    """Energy per site, |M| per site, specific heat, susceptibility, Binder."""
    T = np.asarray(temperatures, dtype=np.float64)
    N = L * L
    E = np.asarray(samples["energy"], dtype=np.float64)
    M = np.asarray(samples["magnetization"], dtype=np.float64)
    moments = {"E": E, "E2": E ** 2, "M": M, "absM": np.abs(M), "M2": M ** 2, "M4": M ** 4}

    def est(m):
        return np.stack((m["E"] / N, m["absM"] / N, (m["E2"] - m["E"] ** 2) / (N * T ** 2),
                         (m["M2"] - m["M"] ** 2) / (N * T), 1 - m["M4"] / (3 * m["M2"] ** 2)))

    value, error = jackknife(moments, est, block_size)
    return dict(zip(("energy", "magnetization", "heat_capacity", "susceptibility", "binder"), zip(value, error)))


def kawamura_observables(samples, L, temperatures, J=1.0, block_size=100):
    """Energy per site, the chirality, phase and spin order parameters and
    the helicity modulus (models/kawamura/analysis.py:33-78 estimators, from
    per-sample squared order parameters over N^2 = L^4)."""
    T = np.asarray(temperatures, dtype=np.float64)
    s = {k: np.asarray(v, dtype=np.float64) for k, v in samples.items()}
    tau2 = s["chirality"] ** 2 / L ** 4
    phase2 = (s["px"] ** 2 + s["py"] ** 2) / L ** 4
    spin2 = s["spin2"] / L ** 4
    moments = {"e": s["energy"] / L ** 2, "tau2": tau2, "phase2": phase2, "spin2": spin2,
               "cx": s["twist_cos_x"], "qx": s["twist_sin_x"], "qx2": s["twist_sin_x"] ** 2}

    def est(m):
        helicity = (J * m["cx"] - J ** 2 / T * (m["qx2"] - m["qx"] ** 2)) / L ** 2
        return np.stack((m["e"], np.sqrt(m["tau2"]), np.sqrt(m["phase2"]), np.sqrt(m["spin2"]), helicity))

    value, error = jackknife(moments, est, block_size)
    return dict(zip(("energy", "chiral_order", "phase_order", "spin_order", "helicity"), zip(value, error)))


def he3_observables(samples, L, temperatures, block_size=100):
    """Energy and density per site, |chirality / density|, phase order, the
    chirality Binder ratio, the mean helicity modulus and Qzz alignment."""
    T = np.asarray(temperatures, dtype=np.float64)
    s = {k: np.asarray(v, dtype=np.float64) for k, v in samples.items()}
    chi = s["chirality"] / s["density"]
    phase2 = (s["phase_real"] ** 2 + s["phase_imag"] ** 2) / L ** 4
    moments = {"energy": s["energy"] / L ** 2, "density": s["density"] / L ** 2, "chirality": np.abs(chi),
               "chi2": chi ** 2, "chi4": chi ** 4, "phase2": phase2, "phase4": phase2 ** 2,
               "kx": s["curvature_x"], "ky": s["curvature_y"], "ix": s["current_x"], "iy": s["current_y"],
               "ix2": s["current_x"] ** 2, "iy2": s["current_y"] ** 2, "qzz": s["spin_alignment"]}

    def est(m):
        hx = (m["kx"] - (m["ix2"] - m["ix"] ** 2) / T) / L ** 2
        hy = (m["ky"] - (m["iy2"] - m["iy"] ** 2) / T) / L ** 2
        return np.stack((m["energy"], m["density"], m["chirality"], np.sqrt(m["phase2"]),
                         1 - m["chi4"] / (3 * m["chi2"] ** 2), 0.5 * (hx + hy), m["qzz"]))

    value, error = jackknife(moments, est, block_size)
    names = ("energy", "density", "chirality", "phase", "binder_chirality", "helicity", "spin_alignment")
    return dict(zip(names, zip(value, error)))


def family_bound(m, n_sigma=3.0):
    """Per-comparison bound for m comparisons whose family-wise two-sided
    false-alarm rate equals that of a single n_sigma test (Bonferroni):
    sqrt(2) * erfcinv(erfc(n_sigma / sqrt(2)) / m), by bisection."""
    target = math.erfc(n_sigma / math.sqrt(2)) / m
    lo, hi = n_sigma, 40.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if math.erfc(mid / math.sqrt(2)) > target:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def n_comparisons(a):
    return sum(np.atleast_1d(v[0]).size for v in a.values())


def compare(a, b, n_sigma=3.0):
    """Observables of two runs that differ by more than ``n_sigma`` combined
    standard errors: list of (name, index, a, b, sigma)."""
    bad = []
    for name in a:
        va, ea = (np.atleast_1d(x) for x in a[name])
        vb, eb = (np.atleast_1d(x) for x in b[name])
        sig = np.sqrt(ea ** 2 + eb ** 2)
        for k in np.nonzero(np.abs(va - vb) > n_sigma * sig)[0]:
            bad.append((name, int(k), float(va[k]), float(vb[k]), float(sig[k])))
    return bad
