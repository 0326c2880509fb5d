"""XY, Kawamura and He3 CUDA kernels: reference-test ports and oracle parity.

Continuous-spin updates match the oracle per site within float32 rounding
(1e-5 absolute); an accept/reject decision may differ only where the
uniform lies within rounding of the acceptance probability, so at most a
tiny fraction of sites may disagree.  RNG states must match bit for bit
(every kernel takes exactly the reference's draws per visit).
"""

import numpy as np
import pytest

import npref
import oracle

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-5
MAX_FLIP_FRACTION = 1e-3


def assert_rng_equal(device_states, host_states):
    got = device_states.copy_to_host()
    np.testing.assert_array_equal(got["s0"], host_states[:, 0])
    np.testing.assert_array_equal(got["s1"], host_states[:, 1])


def assert_states_close(got, ref, per_site_axes):
    diff = np.abs(got.astype(np.complex128) - ref.astype(np.complex128))
    if per_site_axes:
        diff = diff.max(axis=per_site_axes)
    bad = diff > STATE_TOL
    assert bad.mean() <= MAX_FLIP_FRACTION, f"{bad.sum()} of {bad.size} sites differ"


# ------------------------------------------------------------------ XY

def test_xy_ordered_measurements_include_coupling():
    """tests/test_simulation.py:25-41."""
    from mcgb.core.runtime import Runtime
    from mcgb.models.xy.model import XYModel
    model = XYModel(J=1.37)
    rt = Runtime(model, L=4, temperatures=[0.8, 1.0])
    m = rt.measure()
    expected = {"energy": -2 * model.J * 16, "mx": 16, "my": 0, "twist_cos_x": 16, "twist_sin_x": 0}
    assert m.keys() == expected.keys()
    for name, value in expected.items():
        assert m[name].shape == (2,) and m[name].dtype == np.float64
        np.testing.assert_allclose(m[name], value, atol=1e-12)


@pytest.mark.parametrize("L", [4, 6, 32])
def test_xy_measure_matches_complex_bonds(L):
    """tests/test_simulation.py:43-70."""
    from mcgb import device
    from mcgb.models.xy.model import XYModel
    model = XYModel(J=1.37)
    ang = np.random.default_rng(17).uniform(-np.pi, np.pi, (3, L, L)).astype(np.float32)
    m = model.measure(device.to_device(ang))
    for name, values in npref.xy(ang, model.J).items():
        np.testing.assert_allclose(m[name], values, rtol=1e-12, atol=1e-10)


@pytest.mark.parametrize("proposal", ["uniform", "gaussian"])
def test_xy_one_sweep_matches_oracle(proposal):
    from mcgb import device
    from mcgb.core.runtime import Runtime
    from mcgb.models.xy.model import XYModel
    L, T = 32, [0.7, 0.9, 1.1, 1.2]
    sig = np.array([0.9, 1.1, 1.4, 1.6], np.float32)
    model = XYModel(J=1.0, proposal=proposal, sigmas=device.to_device(sig) if proposal == "gaussian" else None)
    rt = Runtime(model, L, T, seed=5)
    ang = np.random.default_rng(6).uniform(-np.pi, np.pi, (4, L, L)).astype(np.float32)
    rt.state.copy_to_device(ang)
    rt.sweep()
    ref, ref_rng = ang.copy(), oracle.rng_states(4 * L * L, 5)
    betas = (1 / np.array(T)).astype(np.float32)
    for c in range(4):
        if proposal == "uniform":
            oracle.xy_update_color(ref, ref_rng, betas, c, np.float32(1), np.float32(1.5))
        else:
            oracle.xy_update_color_gauss(ref, ref_rng, betas, sig, c, np.float32(1))
    assert_rng_equal(rt.rng_states, ref_rng)
    assert_states_close(rt.snapshot(), ref, None)


def test_xy_plain_fp64_form_energy_and_moves():
    from mcgb import _lib, device
    L, R = 16, 2
    th = np.random.default_rng(3).uniform(-np.pi, np.pi, (R, L, L))
    d_th = device.to_device(th)
    rs = device.DeviceArray((R * L * L,), device.XOROSHIRO128P_DTYPE)
    from mcgb.rng import init_xoroshiro128p_states
    init_xoroshiro128p_states(rs, 11)
    out = device.device_array(R, np.float64)
    for r in range(R):
        _lib.call("mcgb_xy64_energy", d_th.cptr, R, L, r, 1.0, out.cptr, _lib.stream_handle())
    np.testing.assert_allclose(out.copy_to_host(), npref.xy(th, 1.0)["energy"], rtol=1e-12, atol=1e-10)
    betas = device.to_device(np.zeros(R))
    for r in range(R):
        for c in range(4):
            _lib.call("mcgb_xy64_update_color", d_th.cptr, rs.cptr, betas.cptr, None, None, R, L, r, c, 1.0, 1.5,
                      _lib.stream_handle())
    moved = d_th.copy_to_host()
    assert np.all(moved != th) and np.all(np.abs(moved) <= np.pi)


# ------------------------------------------------------------------ Kawamura

def test_kawamura_ordered_energy_and_observables():
    """tests/test_kawamura.py:62-71."""
    from mcgb.core.runtime import Runtime
    from mcgb.models.kawamura.model import KawamuraModel
    model = KawamuraModel(J=1.37)
    rt = Runtime(model, 4, [0.6, 0.9], threads=2)
    m = rt.measure()
    expected = {"energy": -4 * float(model.J) * 16, "chirality": 16, "px": 16, "py": 0,
                "spin2": 2 * 16**2 / 9, "twist_cos_x": 32, "twist_sin_x": 0}
    for name, value in expected.items():
        np.testing.assert_allclose(m[name], value, atol=1e-12)
    assert rt.snapshot().dtype == np.float32


@pytest.mark.parametrize("L", [4, 6, 20])
def test_kawamura_measurements_energy_and_order(L):
    """tests/test_kawamura.py:79-94."""
    from mcgb import device
    from mcgb.models.kawamura.model import KawamuraModel
    model = KawamuraModel(J=1.37)
    st = npref.random_kawamura(np.random.default_rng(63), 3, L)
    d = device.to_device(st)
    ref = npref.kawamura(st, model.J)
    m = model.measure(d)
    for name in ref:
        np.testing.assert_allclose(m[name], ref[name], atol=1e-10, rtol=1e-12)
    e = device.device_array(3, np.float64)
    model.measure_energy(d, e)
    np.testing.assert_allclose(e.copy_to_host(), ref["energy"], atol=1e-10)
    order = np.array([2, 0, 1], np.int32)
    o = model.measure(d, device.to_device(order))
    for name in ref:
        np.testing.assert_allclose(o[name][order], ref[name], atol=1e-10)


def test_kawamura_local_energy_changes_match_total_hamiltonian():
    """tests/test_kawamura.py:96-115."""
    from mcgb import device
    from mcgb.models.kawamura.model import KawamuraModel
    model = KawamuraModel(J=1.37)
    st = npref.random_kawamura(np.random.default_rng(63), 3, 6)
    d = device.to_device(st)
    old = npref.kawamura(st, model.J)["energy"]
    for field in ("phase", "chirality", "spin"):
        prop = st[:, 1, 2].copy()
        if field == "phase":
            prop[:, 0] += 0.7
        elif field == "chirality":
            prop[:, 1] *= -1
        else:
            prop[:, 2:] = np.array([0.6, 0, 0.8])
        pos = np.array([[r, 1, 2] for r in range(3)], np.int32)
        e = model.local_energies(d, pos, prop)
        changed = st.copy()
        changed[:, 1, 2] = prop
        np.testing.assert_allclose(e[1] - e[0], npref.kawamura(changed, model.J)["energy"] - old,
                                   atol=3e-6, rtol=1e-5)


def test_kawamura_gauge_symmetry():
    """tests/test_kawamura.py:117-126."""
    from mcgb import device
    from mcgb.models.kawamura.model import KawamuraModel
    model = KawamuraModel()
    st = npref.random_kawamura(np.random.default_rng(63), 3, 6)
    a = model.measure(device.to_device(st))
    st[:, ::2, ::2, 0] += np.float32(np.pi)
    st[:, ::2, ::2, 2:] *= -1
    b = model.measure(device.to_device(st))
    for name in a:
        np.testing.assert_allclose(b[name], a[name], atol=1e-5)


def test_kawamura_hot_and_cold_limits():
    """tests/test_kawamura.py:128-143 (tau parity is deterministic at beta = 0)."""
    from mcgb.core.runtime import Runtime
    from mcgb.models.kawamura.model import KawamuraModel
    rt = Runtime(KawamuraModel(), 6, [0.6, 1.0], threads=2)
    rt.betas.copy_to_device(np.zeros(2, np.float32))
    for _ in range(20):
        rt.sweep()
    st = rt.snapshot()
    assert np.all(np.abs(st[..., 0]) <= np.pi + 1e-6)
    assert set(np.unique(st[..., 1])) == {1.0}
    np.testing.assert_allclose(np.linalg.norm(st[..., 2:], axis=-1), 1, atol=2e-6)
    assert np.std(st[..., 0]) > 0.1 and np.std(st[..., 2:]) > 0.1
    rt.sweep()
    assert set(np.unique(rt.snapshot()[..., 1])) == {-1.0}
    cold = Runtime(KawamuraModel(), 4, [0.6, 1.0], threads=2)
    cold.betas.copy_to_device(np.full(2, 1e8, np.float32))
    for _ in range(4):
        cold.sweep()
    np.testing.assert_allclose(cold.measure()["energy"], -64, atol=1e-5)


def test_kawamura_one_sweep_matches_oracle():
    from mcgb.core.runtime import Runtime
    from mcgb.models.kawamura.model import KawamuraModel
    L, T = 20, [0.65, 0.7, 0.8]
    rt = Runtime(KawamuraModel(), L, T, seed=8)
    st = npref.random_kawamura(np.random.default_rng(9), 3, L)
    rt.state.copy_to_device(st)
    rt.sweep()
    ref, rr = st.copy(), oracle.rng_states(3 * L * L, 8)
    betas = (1 / np.array(T)).astype(np.float32)
    for c in range(4):
        oracle.kawamura_update_color(ref, rr, betas, c, np.float32(1), np.float32(1.5))
    assert_rng_equal(rt.rng_states, rr)
    assert_states_close(rt.snapshot(), ref, -1)


# ------------------------------------------------------------------ He3

def he3_coeffs(pressure=None, reduced_temperature=1.0):
    from mcgb.models.he3.model import He3Model
    return He3Model(pressure=pressure, reduced_temperature=reduced_temperature).betas


def test_he3_coefficients_match_published_table():
    """tests/test_he3.py:87-117 (CPU-side, run here for completeness)."""
    from mcgb.models.he3.model import He3Model
    weak = np.array([-0.5, 1, 1, 1, -1])
    np.testing.assert_array_equal(He3Model().betas, weak.astype(np.float32))
    full = np.asarray(He3Model(pressure=20).betas)
    half = np.asarray(He3Model(pressure=20, reduced_temperature=0.5).betas)
    np.testing.assert_allclose(half - weak, 0.5 * (full - weak), atol=1e-7, rtol=0)


def test_he3_ordered_state_and_normalisations():
    """tests/test_he3.py:127-145."""
    from mcgb.core.runtime import Runtime
    from mcgb.models.he3.model import He3Model
    K, betas = 1.3, (-0.5, 1.0, 1.0, 1.0, -1.0)
    rt = Runtime(He3Model(K=K, betas=betas), 4, [0.6, 0.9], threads=2)
    st = rt.snapshot()
    assert st.dtype == np.complex64
    B = sum(betas[i] for i in (1, 3, 4))
    n = float(np.sum(np.abs(st[0, 0, 0].astype(np.complex128))**2))
    np.testing.assert_allclose(n, 1 / B, atol=1e-7)
    m = rt.measure()
    expected = {"energy": -2 * n * 16 + B * n**2 * 16, "density": n * 16, "chirality": n * 16,
                "phase_real": n * 16, "phase_imag": 0, "current_x": 0, "current_y": 0,
                "curvature_x": 4 * float(np.float32(K)) * n * 16,
                "curvature_y": 4 * float(np.float32(K)) * n * 16, "spin_alignment": 1}
    for name, value in expected.items():
        np.testing.assert_allclose(m[name], value, atol=1e-6)


@pytest.mark.parametrize("L", [4, 6, 20, 80])
def test_he3_measurements_total_energy_and_order(L):
    """tests/test_he3.py:155-180."""
    from mcgb import device
    from mcgb.models.he3.model import He3Model
    K = np.float32(0.73)
    betas = np.asarray((-0.4, 1.1, 0.8, 1.3, -0.7), np.float32)
    model = He3Model(K=K, betas=betas)
    st = npref.random_he3(np.random.default_rng(253), (3, L, L, 3, 2))
    d = device.to_device(st)
    ref = npref.he3(st, float(K), betas.astype(float))
    m = model.measure(d)
    for name in ref:
        budget = (8 if name == "energy" else 2) * np.finfo(np.float32).eps
        np.testing.assert_allclose(m[name] / L**2, ref[name] / L**2, atol=budget, rtol=0, err_msg=name)
    e = device.device_array(3, np.float64)
    model.measure_energy(d, e)
    np.testing.assert_array_equal(e.copy_to_host(), m["energy"])
    cached = model.measure_with_energy(d, e)
    for name in m:
        np.testing.assert_array_equal(cached[name], m[name])
    order = np.array([2, 0, 1], np.int32)
    o = model.measure(d, device.to_device(order))
    for name in m:
        np.testing.assert_array_equal(o[name][order], m[name])


def test_he3_helicity_derivatives():
    """tests/test_he3.py:182-197."""
    from mcgb import device
    from mcgb.models.he3.model import He3Model
    K = np.float32(0.73)
    betas = np.asarray((-0.4, 1.1, 0.8, 1.3, -0.7), np.float32)
    st = npref.random_he3(np.random.default_rng(253), (3, 4, 4, 3, 2))
    m = He3Model(K=K, betas=betas).measure(device.to_device(st))
    h = 2e-4
    e = npref.he3_energy(st, float(K), betas.astype(float))
    for axis, dname in enumerate(("x", "y")):
        tw = np.zeros(2)
        tw[axis] = h
        plus = npref.he3_energy(st, float(K), betas.astype(float), tw)
        minus = npref.he3_energy(st, float(K), betas.astype(float), -tw)
        np.testing.assert_allclose(m[f"current_{dname}"], (plus - minus) / (2 * h), atol=2e-6, rtol=1e-7)
        np.testing.assert_allclose(m[f"curvature_{dname}"], (plus - 2 * e + minus) / h**2, atol=2e-5, rtol=1e-6)


@pytest.mark.parametrize("L", [4, 6, 20])
@pytest.mark.parametrize("pressure", [None, 0.0, 20.0, 34.0])
def test_he3_direct_differences_match_full_change(L, pressure):
    """tests/test_he3_energy_difference.py:137-160, 305-322."""
    from mcgb import device
    from mcgb.models.he3.model import He3Model
    model = He3Model(K=0.73, pressure=pressure)
    rng = np.random.default_rng(20261027)
    pos = np.array([(0, 0), (0, L - 1), (L - 1, 0), (L - 1, L - 1), (0, L // 2), (L // 2, 0),
                    (L - 1, L // 2), (L // 2, L - 1), (1, 1), (1, 2), (2, 1), (2, 2)], np.int32)
    st = npref.random_he3(rng, (len(pos), L, L, 3, 2))
    old = np.stack([st[r, i, j] for r, (i, j) in enumerate(pos)])
    prop = np.empty_like(old)
    prop.real = old.real + rng.uniform(-0.15, 0.15, size=old.shape).astype(np.float32)
    prop.imag = old.imag + rng.uniform(-0.15, 0.15, size=old.shape).astype(np.float32)
    rows = np.array([(r, i, j) for r, (i, j) in enumerate(pos)], np.int32)
    meas = model.local_differences(device.to_device(st), rows, prop, g_d=0.0)
    changed = st.copy()
    for r, (i, j) in enumerate(pos):
        changed[r, i, j] = prop[r]
    ov, og = npref.he3_energy_parts(st, model.betas)
    nv, ng = npref.he3_energy_parts(changed, model.betas)
    K = float(model.K)
    np.testing.assert_allclose(meas[0], ng - og, rtol=3e-6, atol=6e-6)
    _, os_ = npref.he3_potential(old, model.betas)
    _, ns_ = npref.he3_potential(prop, model.betas)
    eps = np.finfo(np.float32).eps
    pb = 8 * eps * np.maximum(1, os_ + ns_)
    np.testing.assert_array_less(np.abs(meas[1] - (nv - ov)), pb)
    gb = 6e-6 + 3e-6 * np.abs(ng - og)
    tb = pb + K * gb + 2 * eps * (np.abs(nv - ov) + np.abs(K * (ng - og)))
    np.testing.assert_array_less(np.abs(meas[2] - (nv - ov + K * (ng - og))), tb)


def test_he3_spin_alignment_normalisation():
    """tests/test_he3.py:238-251."""
    from mcgb import device
    from mcgb.models.he3.model import He3Model
    st = np.zeros((5, 4, 4, 3, 2), np.complex64)
    orb = np.array([1, 1j], np.complex64) / np.sqrt(2)
    st[0, ..., 2, :] = orb
    st[1, ..., 0, :] = orb
    st[2] = np.ones((3, 1)) * orb / np.sqrt(3)
    st[3, :2, :, 2, :] = np.sqrt(3) * orb
    st[3, 2:, :, 0, :] = orb
    m = He3Model(g_d=0.001).measure(device.to_device(st))
    np.testing.assert_allclose(m["spin_alignment"], [1, -0.5, 0, 0.625, 0], atol=1e-7, rtol=0)


@pytest.mark.parametrize("gaussian", [False, True])
def test_he3_one_sweep_matches_oracle(gaussian):
    from mcgb.core.runtime import Runtime
    from mcgb.models.he3.model import He3Model
    from mcgb.models.he3.sampling import He3GaussianRuntime
    L, T = 20, [0.3, 0.4, 0.6]
    model = He3Model(pressure=20, g_d=0.001)
    cls = He3GaussianRuntime if gaussian else Runtime
    rt = cls(model, L, T, threads=2, seed=227)
    st = npref.random_he3(np.random.default_rng(4), (3, L, L, 3, 2))
    rt.state.copy_to_device(st)
    rt.sweep()
    ref, rr = st.copy(), oracle.rng_states(3 * L * L, 227)
    betas = (1 / np.array(T)).astype(np.float32)
    counts = np.zeros((3, 3, L, L), np.int64)
    for c in range(4):
        if gaussian:
            oracle.he3_gaussian_update_color(ref, rr, betas, c, model.betas, model.K, np.float32(-0.9),
                                             np.float32(0), model.g_d, counts)
        else:
            oracle.he3_update_color(ref, rr, betas, c, model.betas, model.K, model.delta, model.g_d)
    assert_rng_equal(rt.rng_states, rr)
    assert_states_close(rt.snapshot(), ref, (-2, -1))
    if gaussian:
        d = rt.sampling_diagnostics()
        assert sum(d["attempts"]) == 3 * L * L and sum(d["nonfinite_rejections"]) == 0
        assert abs(sum(d["accepted"]) - counts[1].sum()) <= MAX_FLIP_FRACTION * counts[0].sum() + 1


def test_he3_hot_moves_and_cold_minimum():
    """tests/test_he3.py:352-366."""
    from mcgb.core.runtime import Runtime
    from mcgb.models.he3.model import He3Model
    rt = Runtime(He3Model(delta=0.15), 6, [0.6, 0.9], threads=2)
    init = rt.snapshot()
    rt.betas.copy_to_device(np.zeros(2, np.float32))
    for _ in range(10):
        rt.sweep()
    st = rt.snapshot()
    assert np.isfinite(st).all() and np.std(st - init) > 0.03
    cold = Runtime(He3Model(delta=0.15), 4, [0.6, 0.9], threads=2)
    e0 = cold.measure()["energy"]
    cold.betas.copy_to_device(np.full(2, 1e8, np.float32))
    for _ in range(4):
        cold.sweep()
    np.testing.assert_allclose(cold.measure()["energy"], e0, atol=1e-5)


@pytest.mark.parametrize("kind", ["ising", "xy", "xy_gauss", "kawamura"])
def test_fused_sweep_equals_four_colour_launches(kind):
    """Runtime.sweep of an unmodified built-in model runs colours 0, {1, 2}, 3
    in three launches (colours 1 and 2 share no bond): bit-identical to the
    reference's four update_color calls, streams included."""
    from mcgb.core.runtime import Runtime
    from mcgb.device import to_device
    from mcgb.models.ising.model import IsingModel
    from mcgb.models.kawamura.model import KawamuraModel
    from mcgb.models.xy.model import XYModel
    R, L, seed = 3, 16, 31
    r = np.random.default_rng(7)
    if kind == "ising":
        make, init = (lambda: IsingModel()), r.choice(np.array([-1, 1], np.int8), (R, L, L))
    elif kind.startswith("xy"):
        sig = to_device(np.array([0.9, 1.2, 1.5], np.float32))
        make = (lambda: XYModel(proposal="gaussian", sigmas=sig)) if kind == "xy_gauss" else (lambda: XYModel())
        init = r.uniform(-np.pi, np.pi, (R, L, L)).astype(np.float32)
    else:
        make = lambda: KawamuraModel()  # noqa: E731
        init = np.zeros((R, L, L, 5), np.float32)
        init[..., 0] = r.uniform(-np.pi, np.pi, (R, L, L))
        init[..., 1] = r.choice([-1.0, 1.0], (R, L, L))
        d = r.normal(size=(R, L, L, 3))
        init[..., 2:] = d / np.linalg.norm(d, axis=-1, keepdims=True)
    T = [0.8, 1.5, 2.5]
    a, b = Runtime(make(), L, T, seed=seed), Runtime(make(), L, T, seed=seed)
    for rt in (a, b):
        rt.state.copy_to_device(init)
    for _ in range(3):
        a.sweep()
        for c in range(4):
            b.model.update_color(b.state, b.rng_states, b.betas, c, b.blocks_per_grid, b.threads_per_block)
    np.testing.assert_array_equal(a.snapshot(), b.snapshot())
    ra, rb = a.rng_states.copy_to_host(), b.rng_states.copy_to_host()
    np.testing.assert_array_equal(ra["s0"], rb["s0"])
    np.testing.assert_array_equal(ra["s1"], rb["s1"])
