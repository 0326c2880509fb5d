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
