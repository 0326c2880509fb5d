"""The shape choice for size groups running side by side (host logic)."""

from mcgb.batch import side_by_side_pick


def test_fastest_shapes_kept_when_they_fit_together():
    # Two groups whose fastest shapes hold half the GPU each: nothing to trade.
    rows = [[(1.0, 0.5), (1.2, 0.3)], [(0.8, 0.4), (0.9, 0.2)]]
    assert side_by_side_pick(rows) == [0, 0]


def test_a_group_gives_up_speed_for_room():
    # Group 0 alone is fastest on the whole GPU (occupancy 1.0); beside group
    # 1 a narrower shape finishes the window sooner: max(1.5, 0.9 + 0.9) = 1.8
    # against max(1.0, 1.0 + 0.9) = 1.9.
    rows = [[(1.0, 1.0), (1.5, 0.9)], [(0.9, 0.9)]]
    assert side_by_side_pick(rows) == [1, 0]


def test_longest_group_bounds_the_window():
    # Shrinking group 1 cannot beat the 2.0 ms of group 0 alone.
    rows = [[(2.0, 1.0)], [(0.5, 0.5), (0.6, 0.1)]]
    assert side_by_side_pick(rows)[0] == 0
    assert max(rows[0][0][0], rows[0][0][1] + rows[1][side_by_side_pick(rows)[1]][1]) == 2.0


class _FakeBatch:
    """The parts of LadderBatch that _refine_side_by_side drives: groups, a
    shape setter and a step timer that reads the configured shapes."""

    def __init__(self, n_groups, step_ms):
        self.groups = list(range(n_groups))
        self.shapes = [None] * n_groups
        self.step_ms = step_ms
        self.timed = []

    def _configure_group(self, g, C, T):
        self.shapes[g] = (C, T)

    def _time_steps(self, n):
        self.timed.append(tuple(self.shapes))
        return self.step_ms(tuple(self.shapes))


def test_refinement_finds_the_shape_that_packs_better():
    from mcgb.batch import LadderBatch
    # Group 1's fastest shape alone (8, 128) packs worse beside group 0 than
    # its runner-up (2, 1024), which real steps reveal.
    per_group = [[(1.0, 8, 1024)], [(0.20, 8, 128), (0.22, 2, 1024), (0.40, 1, 128)]]
    steps = {((8, 1024), (8, 128)): 1.6, ((8, 1024), (2, 1024)): 1.3}
    fake = _FakeBatch(2, lambda sh: steps.get(sh, 9.0))
    shapes, ms = LadderBatch._refine_side_by_side(fake, per_group, [(8, 1024), (8, 128)], 1.6, 10)
    assert shapes == [(8, 1024), (2, 1024)] and ms == 1.3
    assert fake.shapes == [(8, 1024), (2, 1024)]
    # The win was confirmed by timing both again.
    assert fake.timed == [((8, 1024), (2, 1024)), ((8, 1024), (8, 128)), ((8, 1024), (2, 1024))]
    # (1, 128) is beyond the tolerance of group 1's fastest: never timed.
    assert all(sh[1] != (1, 128) for sh in fake.timed)


def test_refinement_rejects_a_win_that_does_not_hold_up():
    from mcgb.batch import LadderBatch
    per_group = [[(1.0, 8, 1024)], [(0.20, 1, 1024), (0.21, 2, 1024)]]
    # (2, 1024) times fast once (noise), then no faster than the incumbent.
    runs = iter([1.40, 1.50, 1.49])
    fake = _FakeBatch(2, lambda sh: next(runs))
    shapes, ms = LadderBatch._refine_side_by_side(fake, per_group, [(8, 1024), (1, 1024)], 1.5, 10)
    assert shapes == [(8, 1024), (1, 1024)] and ms == 1.50
    assert fake.shapes == [(8, 1024), (1, 1024)]


def test_a_win_below_the_margin_is_not_taken():
    from mcgb.batch import LadderBatch
    per_group = [[(1.0, 8, 1024)], [(0.20, 1, 1024), (0.21, 2, 1024)]]
    fake = _FakeBatch(2, lambda sh: 1.48)
    shapes, _ = LadderBatch._refine_side_by_side(fake, per_group, [(8, 1024), (1, 1024)], 1.5, 10)
    assert shapes == [(8, 1024), (1, 1024)] and len(fake.timed) == 1


def test_refinement_keeps_the_shapes_when_nothing_beats_them_and_respects_the_budget():
    from mcgb.batch import LadderBatch
    per_group = [[(1.0, 4, 512), (1.05, 2, 1024), (1.1, 8, 256)], [(0.5, 1, 128), (0.52, 2, 128)]]
    fake = _FakeBatch(2, lambda sh: 2.0)
    shapes, ms = LadderBatch._refine_side_by_side(fake, per_group, [(4, 512), (1, 128)], 1.5, 10, budget=2)
    assert shapes == [(4, 512), (1, 128)] and ms == 1.5
    assert len(fake.timed) == 2
    # The slowest group's runners-up come first.
    assert fake.timed[0][0] == (2, 1024) and fake.timed[1][0] == (8, 256)
    assert fake.shapes == [(4, 512), (1, 128)]
