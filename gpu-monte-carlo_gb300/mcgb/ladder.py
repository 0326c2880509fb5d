"""Temperature ladders for parallel tempering.

``make_temperature_ladder`` follows utils/temperature_ladder.py:5-105: the
ladder is built in inverse temperature, uniform in beta unless ``Tc`` is
given, in which case the beta density is raised smoothly (a tanh shoulder,
1/8 of the window wide) over the temperature window ``Tc +- tc_window/2`` so
that a fraction ``tc_fraction`` of the ladder falls inside it; temperatures
are the equally spaced quantiles of that density, returned in increasing
order.  The same grid (4097 points), integration (trapezoid) and
interpolation steps are used, so ladders agree with the reference's to
rounding.

``ragged_ladders`` builds the per-size ladders of a finite-size study, and
``adapt_ladder`` moves interior temperatures so that neighbouring swap
acceptance rates equalise (a host-side feedback step between runs).
"""

import numpy as np

_GRID = 4097


def _trapezoid(y, x):
    y, x = np.asarray(y, np.float64), np.asarray(x, np.float64)
    return float(np.sum(0.5 * (y[1:] + y[:-1]) * np.diff(x)))


def make_temperature_ladder(T_min, T_max, n_T, Tc=None, tc_window=0.08, tc_fraction=0.60):
    if not (0 < T_min < T_max):
        raise ValueError("Require 0 < T_min < T_max")
    if n_T < 2:
        raise ValueError("Need at least two temperatures")
    b_min, b_max = 1.0 / T_max, 1.0 / T_min
    if Tc is None:
        return (1.0 / np.linspace(b_min, b_max, n_T))[::-1]

    T_lo, T_hi = Tc - tc_window / 2, Tc + tc_window / 2
    if not T_min < T_lo < T_hi < T_max:
        raise ValueError("Focus window must lie inside range")
    if not 0 < tc_fraction < 1:
        raise ValueError("tc_fraction must be between 0 and 1")

    w_lo, w_hi = 1.0 / T_hi, 1.0 / T_lo            # the window in beta
    beta = np.linspace(b_min, b_max, _GRID)
    edge = (w_hi - w_lo) / 8
    bump = 0.5 * (np.tanh((beta - w_lo) / edge) - np.tanh((beta - w_hi) / edge))

    # density = 1 + a * bump; choose a so that the window holds tc_fraction
    # of the total: (width + a * inside) = tc_fraction * (span + a * total).
    span, width = b_max - b_min, w_hi - w_lo
    total = _trapezoid(bump, beta)
    window = np.r_[w_lo, beta[(beta > w_lo) & (beta < w_hi)], w_hi]
    inside = _trapezoid(np.interp(window, beta, bump), window)
    num, den = tc_fraction * span - width, inside - tc_fraction * total
    if num < -1e-12 or den <= 0:
        raise ValueError("Requested focus fraction is not achievable")
    density = 1.0 + max(0.0, num / den) * bump

    cdf = np.r_[0.0, np.cumsum(0.5 * (density[1:] + density[:-1]) * np.diff(beta))]
    cdf /= cdf[-1]
    return (1.0 / np.interp(np.linspace(0, 1, n_T), cdf, beta))[::-1]


def ragged_ladders(sizes, T_min, T_max, n_T, ladders_per_size=1, **focus):
    """``[(L, temperatures), ...]`` for a finite-size study: every size gets
    ``ladders_per_size`` copies of the same ladder (independent seeds are the
    batch's business), in the order of ``sizes``."""
    T = make_temperature_ladder(T_min, T_max, n_T, **focus)
    return [(int(L), T.copy()) for L in sizes for _ in range(ladders_per_size)]


def adapt_ladder(temperatures, acceptance_rates, strength=1.0):
    """One feedback step towards equal swap acceptance between neighbours.

    Each gap in beta is scaled by (rate / mean rate)**strength -- gaps whose
    pairs swap rarely shrink, easy gaps grow -- then the gaps are renormalised
    so the end temperatures stay fixed.  Pairs that were never attempted
    (rate None or NaN) keep their gap.  Returns increasing temperatures.
    """
    T = np.asarray(temperatures, np.float64)
    if T.ndim != 1 or len(T) < 3 or np.any(T <= 0) or np.any(np.diff(T) <= 0):
        raise ValueError("need at least three increasing positive temperatures")
    rates = np.array([np.nan if r is None else r for r in acceptance_rates], np.float64)
    if rates.shape != (len(T) - 1,):
        raise ValueError("one acceptance rate per neighbouring pair")
    beta = 1.0 / T[::-1]                       # increasing beta
    gaps = np.diff(beta)
    r = rates[::-1]
    known = np.isfinite(r)
    if not known.any():
        return T.copy()
    mean = r[known].mean()
    scale = np.ones_like(gaps)
    scale[known] = (np.clip(r[known], 1e-3, 1.0) / max(mean, 1e-3)) ** strength
    gaps = gaps * scale
    gaps *= (beta[-1] - beta[0]) / gaps.sum()
    new_beta = np.r_[beta[0], beta[0] + np.cumsum(gaps)]
    new_beta[-1] = beta[-1]
    return (1.0 / new_beta)[::-1]
