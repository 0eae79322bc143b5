"""Failure detection on the GPU without a GPU fault.

Every device wait in the engine (an mbarrier completed by a TMA copy or an
MMA) is bounded by the handle's wait_limit_us on the GPU's global timer.
sgfim_selftest_wait launches a kernel whose mbarrier nothing completes, so
its wait runs out: the call must come back with SGFIM_EDEVICE, no copy is in
flight, and the same handle must then count supports exactly as before.
"""
import numpy as np
import pytest

import oracle
from sgfim import _lib, datagen
from sgfim.engine import Engine

pytestmark = pytest.mark.gpu


def _small_case():
    bm = datagen.correlated_bitmaps(20_480, 96, 4, 0.05, 0.4, seed=11)
    cp, ci = datagen.walk_candidates(3_000, 96, 1, 10, seed=12)
    return bm, cp, ci


def test_wait_that_runs_out_returns_edevice_and_handle_stays_usable():
    bm, cp, ci = _small_case()
    want = oracle.support_batch(bm, cp, ci)
    with Engine(device=0, wait_limit_us=2000) as eng:
        eng.load_bitmaps(bm, 20_480)
        assert np.array_equal(eng.support_batch(cp, ci), want)
        assert eng.selftest_wait() == _lib.EDEVICE
        # the error word was read and cleared: later calls are clean and exact
        assert eng.device_status() == 0
        for _ in range(2):
            assert np.array_equal(eng.support_batch(cp, ci), want)
        assert eng.selftest_wait() == _lib.EDEVICE


def test_device_status_clean_after_device_pointer_calls():
    torch = pytest.importorskip("torch")
    bm, cp, ci = _small_case()
    want = oracle.support_batch(bm, cp, ci)
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev).cuda_stream
    tb = torch.from_numpy(bm.view(np.int64)).to(dev)
    tp = torch.from_numpy(cp.view(np.int64)).to(dev)
    ti = torch.from_numpy(ci.view(np.int32)).to(dev)
    out = torch.zeros(len(cp) - 1, dtype=torch.int32, device=dev)
    with Engine(device=0) as eng:
        w = bm.shape[1]
        eng.support_batch_device(tb.data_ptr(), bm.shape[0], w, w, tp.data_ptr(), ti.data_ptr(), len(cp) - 1,
                                 out.data_ptr(), stream)
        assert eng.device_status(stream) == 0
        assert np.array_equal(out.cpu().numpy().view(np.uint32), want)
