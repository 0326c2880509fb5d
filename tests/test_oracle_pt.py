"""The oracle's replica exchange against the reference's PT test expectations
(tests/test_parallel_tempering.py:68-136, :211-253)."""

import numpy as np

import oracle


class PT:
    """Host driver of orc_pt_exchange with the wrapper's schedule."""

    def __init__(self, temperatures, energies, seed=97):
        self.R = len(temperatures)
        self.temperatures = np.asarray(temperatures, float)
        self.betas = (1.0 / self.temperatures).astype(np.float32)
        self.w2t = np.arange(self.R, dtype=np.int32)
        self.t2w = np.arange(self.R, dtype=np.int32)
        self.rng = oracle.rng_states(self.R - 1, seed)
        self.counts = np.zeros((3, self.R - 1), np.int64)
        self.trips = oracle.pt_initial_trips(self.R)
        self.energies = np.asarray(energies, np.float64)
        self.parity = 0
        self.sweeps = 0

    def exchange(self):
        oracle.pt_exchange(self.energies, self.betas, self.w2t, self.t2w, self.rng, self.counts,
                           self.trips, self.parity, self.sweeps)
        if self.R > 2:
            self.parity = 1 - self.parity

    def assert_maps(self, t2w):
        np.testing.assert_array_equal(self.t2w, t2w)
        np.testing.assert_array_equal(self.w2t[self.t2w], np.arange(self.R))
        ladder = (1.0 / self.temperatures).astype(np.float32)
        np.testing.assert_array_equal(self.betas, ladder[self.w2t])


def test_equal_energies_always_swap_and_alternate_parity():
    pt = PT(np.linspace(0.6, 1.4, 4), np.full(4, -10.0))
    pt.exchange()
    pt.assert_maps([1, 0, 3, 2])
    pt.exchange()
    pt.assert_maps([1, 3, 0, 2])
    np.testing.assert_array_equal(pt.counts[:2], [[1, 1, 1], [1, 1, 1]])


def test_odd_and_large_ladders():
    for R in (5, 259):
        pt = PT(np.linspace(0.5, 2.0, R), np.zeros(R))
        order = np.arange(R)
        attempts = np.zeros(R - 1, np.int64)
        for rnd in range(4):
            for t in range(rnd % 2, R - 1, 2):
                order[t:t + 2] = order[t:t + 2][::-1]
                attempts[t] += 1
            pt.exchange()
            pt.assert_maps(order)
            np.testing.assert_array_equal(pt.counts[0], attempts)
            np.testing.assert_array_equal(pt.counts[1], attempts)


def test_nonfinite_energy_blocks_swap_and_is_counted():
    pt = PT([1.0, 2.0], [np.nan, -3.0])
    pt.exchange()
    pt.assert_maps([0, 1])
    assert pt.counts[2, 0] == 1 and pt.counts[0, 0] == 1 and pt.counts[1, 0] == 0


def test_acceptance_sign_uses_current_energies():
    """tests/test_parallel_tempering.py:148-186: cold/low vs hot/high rejects, reverse accepts."""
    mag = 2 * 1.37 * 16
    pt = PT([1e-6, 1e6], [-mag, mag], seed=98)
    pt.exchange()
    pt.assert_maps([0, 1])
    pt.energies = np.array([mag, -mag])
    pt.exchange()
    pt.assert_maps([1, 0])
    np.testing.assert_array_equal(pt.counts[:2, 0], [2, 1])


def test_two_walker_round_trips():
    """tests/test_parallel_tempering.py:211-235 (exchange every 2 sweeps, 6 sweeps)."""
    pt = PT([0.6, 1.4], [0.0, 0.0])
    for sweep in range(1, 7):
        pt.sweeps = sweep
        if sweep % 2 == 0:
            pt.exchange()
    np.testing.assert_array_equal(pt.trips[3], [1, 1])
    np.testing.assert_array_equal(pt.trips[4], [4, 4])


def test_interior_walker_trip_starts_at_first_endpoint():
    """tests/test_parallel_tempering.py:237-253."""
    pt = PT([0.6, 1.0, 1.4], [0.0, 0.0, 0.0])
    for sweep in range(1, 7):
        pt.sweeps = sweep
        pt.exchange()
    np.testing.assert_array_equal(pt.trips[3], [1, 0, 1])
    pt.sweeps = 7
    pt.exchange()
    np.testing.assert_array_equal(pt.trips[3], [1, 1, 1])
    np.testing.assert_array_equal(pt.trips[4], [5, 6, 6])
