"""The plain float64 XY form: its graph replay equals direct launches.

mcgb.plain64.PlainXYLadder is the one-lattice-per-launch float64 baseline of
the mixed-vs-plain comparison; timed, it replays each exchange interval from
a captured CUDA graph with the exchange schedule on a device clock.  The
replay must give exactly the chain of direct launches: angles, streams,
maps, betas and swap/round-trip counters, including partial intervals.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("R,sigmas", [(5, True), (2, False)])
def test_plain_fp64_graph_replay_equals_direct_launches(R, sigmas):
    from mcgb.plain64 import PlainXYLadder
    L, T = 16, np.geomspace(0.7, 1.2, R)
    init = np.random.default_rng(4).uniform(-np.pi, np.pi, (R, L, L))
    sig = np.linspace(0.9, 1.5, R) if sigmas else None
    a = PlainXYLadder(L, T, 21, sigmas=sig, exchange_interval=4, initial_state=init)
    b = PlainXYLadder(L, T, 21, sigmas=sig, exchange_interval=4, initial_state=init)
    for n in (3, 9, 16, 2, 12):
        a.sweep(n, graph=True)
        b.sweep(n, graph=False)
    assert a._graphs, "full intervals were replayed from a graph"
    for _ in range(8):  # sweep by sweep, as simulate() runs its measured sweeps
        a.sweep(1, graph=True)
        b.sweep(1, graph=False)
    for name in ("theta", "rng", "w2t", "t2w", "betas32", "swap_counts", "trips", "energies", "clock"):
        np.testing.assert_array_equal(getattr(a, name).copy_to_host(), getattr(b, name).copy_to_host(),
                                      err_msg=name)
    assert (a.sweeps, a.exchange_rounds, a._parity) == (b.sweeps, b.exchange_rounds, b._parity)
    assert (a.sweeps, a.exchange_rounds) == (50, 12)
    np.testing.assert_array_equal(a.clock.copy_to_host(), [48, 12])
