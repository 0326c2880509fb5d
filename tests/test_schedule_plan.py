"""The Simulation schedule planner against a literal walk of the reference's
host loop (core/simulation.py:39-78 over core/parallel_tempering.py:245-269):
the same exchange rounds (with their sweep numbers and the sweeps since the
previous round), history rows, samples (cached after an exchange or not) and
the same total counts, for every phase of the counters."""

import itertools

import pytest

from mcgb.core.schedule import MAX_COPIES, Segment, chunks, plan


def reference_events(therm, meas, every, interval, start_sweeps, start_rounds, stride):
    """Events in order: ("sweep",), ("exchange", sweep, parity_round), ("record", sweep, round), ("sample", k, cached)."""
    events, sweeps, rounds = [], start_sweeps, start_rounds
    cached = False

    def one_sweep():
        nonlocal sweeps, rounds, cached
        events.append(("sweep",))
        cached = False
        sweeps += 1
        if interval is not None and sweeps % interval == 0:
            events.append(("exchange", sweeps, rounds))
            cached = True
            rounds += 1
            if stride is not None and rounds % stride == 0:
                events.append(("record", sweeps, rounds))

    for _ in range(therm):
        one_sweep()
    for step in range(1, meas + 1):
        one_sweep()
        if step % every == 0:
            events.append(("sample", therm + step, cached))
    return events


def replayed_events(p, start_sweeps, start_rounds):
    events, sweeps, rounds, k = [], start_sweeps, start_rounds, 0
    for seg, count in p.runs:
        for _ in range(count):
            for _ in range(seg.sweeps):
                events.append(("sweep",))
                k += 1
            sweeps += seg.sweeps
            if seg.exchange:
                # the device clock: the round runs after (previous round's sweep + advance) sweeps
                events.append(("exchange", sweeps, rounds))
                rounds += 1
                if seg.record:
                    events.append(("record", sweeps, rounds))
            if seg.sample:
                events.append(("sample", k, seg.exchange))
    return events


@pytest.mark.parametrize("therm,meas,every,interval,start,stride", [
    (0, 1, 1, None, 0, None), (7, 40, 2, None, 0, None), (6, 12, 3, 2, 0, 2), (4, 8, 2, 2, 0, 1),
    (7, 40, 2, 3, 0, None), (13, 37, 5, 4, 3, 3), (0, 100, 10, 10, 25, 10), (5, 23, 23, 7, 1, None),
    (100, 1000, 1, 10, 0, 5), (3, 9, 4, 1, 0, 1),
])
def test_plan_reproduces_the_reference_loop(therm, meas, every, interval, start, stride):
    start_rounds = start // interval if interval else 0
    ref = reference_events(therm, meas, every, interval, start, start_rounds, stride)
    p = plan(therm, meas, every, interval, start, start_rounds, stride)
    assert replayed_events(p, start, start_rounds) == ref
    assert p.n_sweeps == therm + meas
    assert p.sample_sweeps == [e[1] for e in ref if e[0] == "sample"]
    assert p.history == [(e[1], e[2]) for e in ref if e[0] == "record"]
    assert p.n_rounds == sum(e[0] == "exchange" for e in ref)
    assert p.ends_with_exchange == (ref[-1][0] in ("exchange", "record") or
                                    (ref[-1][0] == "sample" and ref[-1][2]))
    # Advances: each round's sweep minus the previous round's (or the start).
    last, got = start, []
    for seg, count in p.runs:
        for _ in range(count):
            if seg.exchange:
                got.append(seg.advance)
    want = []
    for e in ref:
        if e[0] == "exchange":
            want.append(e[1] - last)
            last = e[1]
    assert got == want


def test_periodic_schedules_compress_to_few_segments():
    p = plan(5000, 20000, 10, 10, 0, 0, None)
    assert len(p.runs) <= 3
    assert p.runs[-1] == (Segment(10, True, 10, False, True), 2000)


@pytest.mark.parametrize("n", [1, 2, 3, 63, 64, 65, 200, 1000])
def test_chunks_cover_counts_with_bounded_graph_sizes(n):
    c = chunks(n)
    assert sum(c) == n and all(x <= MAX_COPIES and x & (x - 1) == 0 for x in c)
    assert c == sorted(c, reverse=True)


def test_plan_of_every_small_schedule_matches():
    for therm, meas, every, interval in itertools.product(range(3), range(1, 7), range(1, 4), (None, 1, 2, 3)):
        if every > meas:
            continue
        ref = reference_events(therm, meas, every, interval, 0, 0, 2 if interval else None)
        p = plan(therm, meas, every, interval, 0, 0, 2 if interval else None)
        assert replayed_events(p, 0, 0) == ref, (therm, meas, every, interval)
