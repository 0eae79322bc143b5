"""The allocation-free support entry point against the allocating one.

sgfim_support_batch_noalloc serves callers that may not allocate device
memory (their own pool owns the GPU, or cudaMalloc's synchronisation is not
allowed on their path); it keeps its scratch in a fixed array inside the
library.  This test calls it through the C ABI twice in a row on different
inputs -- so leftovers of the first call in the shared scratch would show --
and requires the same supports as sgfim_support_batch_device and as the CPU
oracle (integer counts: exact equality), with a clean device status
(sgfim_noalloc_status) after each call.  It builds its own inputs and handle,
so it passes alone in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_inputs(torch, dev, seed, n_txn, d, n_cand, kmin, kmax):
    from sgfim import datagen
    bm = datagen.correlated_bitmaps(n_txn, d, 8, 0.02, 0.3, seed=seed)
    cp, ci = datagen.walk_candidates(n_cand, d, kmin, kmax, seed=seed + 100)
    return (torch.from_numpy(bm.view(np.int64)).to(dev), bm.shape[1],
            torch.from_numpy(cp.view(np.int64)).to(dev), torch.from_numpy(ci.view(np.int32)).to(dev), len(cp) - 1,
            (bm, cp, ci))


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    torch = pytest.importorskip("torch")
    import oracle
    from sgfim import _lib
    from sgfim.engine import Engine
    L = _lib.load()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    eng = Engine(device=0)
    try:
        # second call: fewer candidates, other shapes, and k up to 12 (the >8-item list)
        for seed, n_txn, d, n_cand, kmin, kmax in [(3, 64 * 1024, 256, 60_000, 3, 8),
                                                    (4, 16 * 1024, 600, 9_000, 1, 12)]:
            tb, w, tp, ti, n, host = _device_inputs(torch, dev, seed, n_txn, d, n_cand, kmin, kmax)
            ref = torch.zeros(n, dtype=torch.int32, device=dev)
            got = torch.full((n,), -1, dtype=torch.int32, device=dev)
            eng.support_batch_device(tb.data_ptr(), d, w, w, tp.data_ptr(), ti.data_ptr(), n, ref.data_ptr(),
                                     stream)
            rc = L.sgfim_support_batch_noalloc(C.c_void_p(tb.data_ptr()), d, w, w, C.c_void_p(tp.data_ptr()),
                                               C.c_void_p(ti.data_ptr()), n, C.c_void_p(got.data_ptr()),
                                               C.c_void_p(stream))
            assert rc == 0
            assert L.sgfim_noalloc_status(C.c_void_p(stream)) == 0
            torch.cuda.synchronize()
            assert torch.equal(got, ref), f"call with seed {seed} differs"
            want = oracle.support_batch(*host)
            assert np.array_equal(got.cpu().numpy().view(np.uint32), want), f"call with seed {seed} != oracle"
    finally:
        eng.close()


def test_noalloc_rejects_more_than_its_capacity():
    from sgfim import _lib
    L = _lib.load()
    dummy = C.c_void_p(16)
    rc = L.sgfim_support_batch_noalloc(dummy, 4, 2, 2, dummy, dummy, _lib.NOALLOC_MAX_CAND + 1, dummy, None)
    assert rc == _lib.ECAPACITY
