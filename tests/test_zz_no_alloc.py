"""The allocation-free window + exchange entry point.

Callers that cannot allocate device memory (a program inside a host runtime
that owns every device allocation, or a latency-critical loop that cannot
take cudaMalloc's implicit device synchronisation) use
mcgb_batch_window_exchange_noalloc, whose deferred-sample scratch is a fixed
array inside the library.  Two identical batches advance side by side,
one through the existing two calls with caller-allocated scratch and one
through the new entry point; after each of two calls in a row their states,
samples, maps, counters and energies must agree exactly (the same kernels run
on the same inputs).  This file sorts last so a stop-at-first-failure run has
already run every other test.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_batch():
    from mcgb.batch import LadderBatch
    from mcgb.models.xy.model import XYModel
    b = LadderBatch(XYModel(), [(16, np.geomspace(0.7, 1.2, 6)), (32, np.geomspace(0.8, 1.1, 4))],
                    seeds=[11, 12], exchange_interval=5, proposal="gaussian", sigma0=1.2,
                    cluster_size=2, threads=128)
    # Samples every 5 sweeps, so every window ends on a sample that the
    # exchange scatters from the scratch buffer.
    b.allocate_samples(first_sample_sweep=5, sample_interval=5, n_slots=4)
    return b


def two_call_path(b):
    from mcgb import _lib
    s = _lib.stream_handle()
    w = b._window(5, staging=True)
    _lib.call("mcgb_batch_window_run", b.model_id, ctypes.byref(w), s)
    _lib.call("mcgb_batch_exchange", ctypes.byref(w), ctypes.byref(b._pt()), s)
    _lib.call("mcgb_batch_clock_tick", b.clock.cptr, 5, 1, s)


def noalloc_path(b):
    from mcgb import _lib
    s = _lib.stream_handle()
    w = b._window(5, staging=False)
    assert w.staging is None
    _lib.call("mcgb_batch_window_exchange_noalloc", b.model_id, ctypes.byref(w), ctypes.byref(b._pt()), s)
    _lib.call("mcgb_batch_clock_tick", b.clock.cptr, 5, 1, s)


def test_noalloc_window_matches_two_call_path_twice():
    ref, got = make_batch(), make_batch()
    for call in range(2):
        two_call_path(ref)
        noalloc_path(got)
        for name in ("state", "aux", "rng", "betas", "w2t", "t2w", "energies", "e_run", "accepted",
                     "swap_counts", "trips", "samples", "clock"):
            a = getattr(ref, name).copy_to_host()
            b = getattr(got, name).copy_to_host()
            np.testing.assert_array_equal(b, a, err_msg=f"{name} after call {call + 1}")
    # The window-end samples went through the scratch buffer: slots 0 and 1
    # hold finite values in temperature order.
    data = got.samples.copy_to_host()
    assert np.all(np.isfinite(data[:2])) and np.any(data[:2] != 0)


def test_noalloc_window_rejects_oversized_batches_and_caller_scratch():
    from mcgb import _lib
    b = make_batch()
    w = b._window(5, staging=True)
    with pytest.raises(ValueError, match="staging must be NULL"):
        _lib.call("mcgb_batch_window_exchange_noalloc", b.model_id, ctypes.byref(w), ctypes.byref(b._pt()),
                  _lib.stream_handle())
    w = b._window(5, staging=False)
    w.n_replicas = 7000  # 7000 x 5 channels > 32768 (checked before any launch)
    with pytest.raises(ValueError, match="exceed the fixed scratch"):
        _lib.call("mcgb_batch_window_exchange_noalloc", b.model_id, ctypes.byref(w), ctypes.byref(b._pt()),
                  _lib.stream_handle())


def test_noalloc_window_rejects_size_group_windows():
    # A window over one size group covers part of the table; the exchange
    # would then read scratch entries of other replicas that this call never
    # wrote, so the entry point refuses it before any launch.
    from mcgb import _lib
    b = make_batch()
    work = np.arange(6, dtype=np.int32)
    w = b._window(5, staging=False)
    w.host_work_idx = work.ctypes.data
    w.n_work = len(work)
    with pytest.raises(ValueError, match="whole replica table"):
        _lib.call("mcgb_batch_window_exchange_noalloc", b.model_id, ctypes.byref(w), ctypes.byref(b._pt()),
                  _lib.stream_handle())
    w = b._window(5, staging=False)
    w.hold_clock = 1
    with pytest.raises(ValueError, match="hold_clock must be 0"):
        _lib.call("mcgb_batch_window_exchange_noalloc", b.model_id, ctypes.byref(w), ctypes.byref(b._pt()),
                  _lib.stream_handle())
