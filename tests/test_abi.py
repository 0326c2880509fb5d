"""The C ABI: every function include/mcgb.h declares is exported by
libmcgb.so and bound by the ctypes layer; no GPU needed (no compute calls)."""

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "mcgb.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:mcgb|mc)_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from mcgb import _lib
    return _lib.load()


def test_header_declares_the_entry_points():
    names = declared_functions()
    assert "mcgb_rng_init" in names and "mcgb_batch_window_run" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(lib):
    from mcgb import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.lib_path())], capture_output=True, text=True)
    exported = set(re.findall(r"\bT ((?:mcgb|mc)_[a-z0-9_]+)$", out.stdout, flags=re.M))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"


def test_ctypes_layer_binds_every_declared_symbol(lib):
    from mcgb import _lib
    bound = set(_lib.SIGNATURES) | {"mcgb_last_error", "mcgb_version"}
    missing = [n for n in declared_functions() if n not in bound]
    assert not missing, f"declared but not bound in mcgb._lib: {missing}"
    for name in declared_functions():
        assert getattr(lib, name) is not None


def test_argument_validation_without_a_gpu(lib):
    """Invalid sizes are rejected on the host before any CUDA call."""
    from mcgb import _lib
    assert lib.mcgb_ising_update_color(None, None, None, 1, 5, 0, ctypes.c_float(1.0), None) == _lib.EINVAL
    assert "L must be even" in _lib.last_error()
    assert lib.mcgb_pt_exchange(None, None, None, None, None, None, None, 1, 0, 0, None) == _lib.EINVAL
    assert lib.mcgb_batch_channels(1) == 5 and lib.mcgb_batch_channels(4) == 10
    assert lib.mcgb_batch_channels(9) == _lib.EINVAL
    assert lib.mcgb_version().decode().startswith("mcgb")
    # handle API: rejected before any allocation
    h = ctypes.c_void_p()
    params = _lib.MCParams(J=1.0, delta=1.5)
    Ls = (ctypes.c_int32 * 2)(16, 16)
    temps = (ctypes.c_double * 2)(1.0, 2.0)
    assert lib.mc_create(9, ctypes.byref(params), Ls, 2, temps, 1, None, ctypes.byref(h)) == _lib.EINVAL
    assert "per-colour form" in _lib.last_error() and not h.value
    assert lib.mc_create(0, ctypes.byref(params), Ls, 0, temps, 1, None, ctypes.byref(h)) == _lib.EINVAL
    assert lib.mc_get_error(None) == _lib.EINVAL and lib.mc_destroy(None) == 0
    assert lib.mc_sweep(None, 1) == _lib.EINVAL


def test_window_sweep_limits_without_a_gpu(lib):
    """A window of more than 2^24 sweeps, a sample interval above 2^24 and a
    resident launch of more than 2^28 sweeps are refused on the host before
    any CUDA call (the kernels count down to the next sample in an int)."""
    import numpy as np

    from mcgb import _lib
    from mcgb.batch import REPLICA_DTYPE, BatchPT, BatchWindow
    table = np.array([(16, 0, 0, 1, 0)], dtype=REPLICA_DTYPE)
    w = BatchWindow()
    # Device pointers are never dereferenced: the checks run first.
    for name in ("table", "work_ptr", "work_idx", "state", "rng", "aux", "betas", "w2t", "e_run", "energies",
                 "accepted", "clock"):
        setattr(w, name, 256)
    w.host_table = table.ctypes.data
    w.n_replicas = w.n_clusters = w.cluster_size = 1
    w.threads, w.J = 64, 1.0
    w.n_sweeps = (1 << 24) + 1
    assert lib.mcgb_batch_window_run(0, ctypes.byref(w), None) == _lib.EINVAL
    assert "n_sweeps must be in [0, 16777216]" in _lib.last_error()
    w.n_sweeps = 10
    w.samples, w.n_slots, w.n_temps_total, w.sample_interval = 256, 1, 1, (1 << 24) + 1
    assert lib.mcgb_batch_window_run(0, ctypes.byref(w), None) == _lib.EINVAL
    assert "bad sample buffer" in _lib.last_error()
    w.samples, w.sample_interval = None, 0
    w.n_sweeps = 1 << 23
    pt = BatchPT()
    sync = (ctypes.c_int32 * 8)()
    assert lib.mcgb_batch_run_resident(0, ctypes.byref(w), ctypes.byref(pt), sync, 64, None) == _lib.EINVAL
    assert "sweeps a launch" in _lib.last_error()
