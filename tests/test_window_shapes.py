"""Cluster shapes of the window launches (host logic, no GPU)."""

import pytest

from mcgb.batch import LadderBatch
from mcgb.core.window_sweeps import MAX_PLAQUETTES, _shape


@pytest.mark.parametrize("L,C,expected", [(4, 16, 2), (12, 16, 6), (64, 4, 4), (64, 16, 16), (96, 16, 16),
                                          (10, 4, 1), (20, 4, 2), (128, 5, 4), (2048, 16, 16)])
def test_effective_cluster_is_the_largest_divisor_of_the_plaquette_rows(L, C, expected):
    got = LadderBatch.effective_cluster(L, C)
    assert got == expected
    assert (L // 2) % got == 0 and got <= C


@pytest.mark.parametrize("L", [4, 8, 16, 32, 48, 64, 96, 128, 256])
def test_reference_layout_window_shape_holds_one_plaquette_per_thread(L):
    C, T = _shape(L)
    Ce = LadderBatch.effective_cluster(L, C)
    npl = (L // 2) * (L // 2) // Ce
    assert npl <= MAX_PLAQUETTES and npl <= T
    assert T % 32 == 0 and 64 <= T <= 1024
    # The fewest CTAs that do it: one cluster size down would not.
    smaller = [c for c in (1, 2, 4, 8, 16) if c < C]
    if smaller:
        c = smaller[-1]
        assert (L // 2) * (L // 2) // LadderBatch.effective_cluster(L, c) > MAX_PLAQUETTES


def test_reference_layout_window_declines_lattices_beyond_sixteen_ctas():
    # 16 CTAs hold at most 16 x 1024 plaquettes of a colour (L = 256); a larger
    # lattice runs the colour launches instead.
    assert _shape(256) is not None
    assert _shape(512) is None
