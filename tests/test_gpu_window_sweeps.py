"""Runs of drop-in sweeps as one window launch (mcgb/core/window_sweeps.py).

Runtime._enqueue_sweeps(n) runs n sweeps of the built-in Ising plugin, or of
the XY plugin with the reference's uniform proposal, as one window launch of
the batched engine on the Runtime's reference-layout arrays.  It must leave
the lattice and every RNG stream bit-identical to n sweeps of the per-colour
launches (Runtime.sweep), for lattices held by one CTA, by clusters of
several, by clusters whose size does not divide the plaquette rows (L=130:
13 of 16 CTAs hold rows), with more replicas than co-resident clusters, and
for several runs in a row; Gaussian XY proposals and lattices too large for
16 CTAs keep the colour launches.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(kind, R, L, seed, **model_kw):
    from mcgb.core.runtime import Runtime
    r = np.random.default_rng(seed)
    if kind == "ising":
        from mcgb.models.ising.model import IsingModel
        model, T = IsingModel(**model_kw), np.geomspace(1.8, 3.0, R)
        init = r.choice(np.array([-1, 1], np.int8), (R, L, L))
    else:
        from mcgb.models.xy.model import XYModel
        model, T = XYModel(**model_kw), np.geomspace(0.6, 1.4, R)
        init = r.uniform(-np.pi, np.pi, (R, L, L)).astype(np.float32)
    rt = Runtime(model, L, T, seed=seed)
    rt.state.copy_to_device(init)
    return rt


@pytest.mark.parametrize("kind", ["ising", "xy"])
@pytest.mark.parametrize("R,L", [(3, 4), (2, 6), (5, 16), (4, 64), (3, 128), (2, 130), (200, 16)])
def test_window_sweeps_equal_colour_launches(kind, R, L):
    ref, got = make(kind, R, L, 17 + L), make(kind, R, L, 17 + L)
    for n in (1, 7, 10):
        for _ in range(n):
            ref.sweep()
        got._enqueue_sweeps(n)
        assert got._window, "the window launch should serve this lattice"
        np.testing.assert_array_equal(got.state.copy_to_host(), ref.state.copy_to_host())
        np.testing.assert_array_equal(got.rng_states.copy_to_host(), ref.rng_states.copy_to_host())


def test_window_sweeps_fall_back_where_they_do_not_apply():
    from mcgb.device import to_device
    g = make("xy", 2, 16, 5, proposal="gaussian", sigmas=to_device(np.array([0.5, 0.9], np.float32)))
    g._enqueue_sweeps(3)
    assert g._window is False
    big = make("ising", 1, 1024, 6)
    big._enqueue_sweeps(1)
    assert big._window is False
