"""Host-side tests that need no GPU: ABI exports, parsers, adapter mirror,
workload generators, and the multi-process sharding of the bench path."""
import json
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from sgfim import datagen, results

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sgfim.h")
ADAPTER_GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "adapter_golden.json")))


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sgfim_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from sgfim import _lib
    L = _lib.load()
    syms = declared_symbols()
    assert len(syms) >= 19
    for s in syms:
        assert hasattr(L, s), f"libsgfim.so does not export {s}"
    assert set(syms) <= set(_lib.SIGNATURES), "ctypes binding misses a declared symbol"
    assert L.sgfim_abi_version() == 3


def test_open_without_gpu_returns_error_code():
    """With no CUDA device the ABI returns an error code instead of crashing."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from sgfim.engine import Engine, SgfimError
    with pytest.raises(SgfimError):
        Engine()


def test_cli_usage_exit_code():
    from sgfim import _lib
    exe = os.path.join(os.path.dirname(_lib.LIB_PATH), "sgfim_tensorfim")
    p = subprocess.run([exe], capture_output=True)
    assert p.returncode == 2 and b"usage" in p.stderr


# ------------------------------------------------------------------ FIMI parsing
def test_parse_fimi_byte_rules(tmp_path):
    p = tmp_path / "x.txt"
    p.write_bytes(b"1 2 3\n\n4 -5 6\n7\t8,9\n  \n10 11")
    rows = oracle.parse_fimi(str(p))
    assert rows == [[1, 2, 3], [], [4, 6], [7, 8, 9], [], [10, 11]]
    p.write_bytes(b"1 2\n3\n")
    assert oracle.parse_fimi(str(p)) == [[1, 2], [3]]
    p.write_bytes(b"1 2\n-3\n")
    assert oracle.parse_fimi(str(p)) == [[1, 2], []]


# ------------------------------------------------------------------ result files (the adapter's format)
def test_result_patterns_equal_reference():
    """The four patterns are the reference adapter's, character for character."""
    assert results.RECORD.pattern == ADAPTER_GOLD["tf_line"]
    assert results.STAGE_HEADER.pattern == ADAPTER_GOLD["af_stage"]
    assert results.COMPUTATION_TIME.pattern == ADAPTER_GOLD["tf_comp"]
    assert results.TOTAL_TIME.pattern == ADAPTER_GOLD["tf_tot"]


def test_read_results_equals_reference_parsers(tmp_path):
    """read_results gives what the reference's parse_tensorfim_results /
    parse_anyfim_results / cumulative_mfis returned on the same texts."""
    p1, p2 = tmp_path / "tf.txt", tmp_path / "af.txt"
    p1.write_text(ADAPTER_GOLD["tf_text"])
    p2.write_text(ADAPTER_GOLD["af_text"])
    tf = results.read_results(str(p1))
    assert sorted([sorted(k), v] for k, v in tf.sets.items()) == ADAPTER_GOLD["tf_parsed"] and not tf.stages
    af = results.read_results(str(p2))
    assert {str(k): sorted([sorted(s), f] for s, f in v) for k, v in af.stages.items()} == ADAPTER_GOLD["af_parsed"]
    assert af.arrays == ADAPTER_GOLD["af_meta"]
    assert {str(k): sorted(sorted(s) for s in v) for k, v in af.cumulative().items()} == ADAPTER_GOLD["cumulative"]
    assert results.timings(ADAPTER_GOLD["tf_text"]) == (0.5, 0.75)


def test_result_paths_follow_the_engines_naming():
    assert results.result_path("tensorfim", "/d/x.txt", 0.03) == "/d/x.txt-0.030000=Results.txt"
    assert results.result_path("anyfim", "/d/x.txt", 12) == "/d/x.txt-12-stages=Results.txt"


def test_generators_shapes_and_determinism():
    a = datagen.regime_txns(1000, 8, 5, 4, 0.3, seed=0)
    b = datagen.regime_txns(1000, 8, 5, 4, 0.3, seed=0)
    assert np.array_equal(a, b) and a.shape == (1000, 8)
    assert (a // 5 == np.arange(8)[None, :]).all()  # one item per sensor
    bm = datagen.correlated_bitmaps(4096, 32, 4, 0.02, 0.2, seed=1)
    dens = np.unpackbits(bm.view(np.uint8), axis=1).mean(axis=1)
    assert bm.shape == (32, 64) and (dens > 0.002).all() and (dens < 0.5).all()
    cp, ci = datagen.walk_candidates(500, 64, 3, 8, seed=2)
    k = np.diff(cp)
    assert k.min() >= 3 and k.max() <= 8
    for c in range(500):
        s = ci[cp[c]:cp[c + 1]]
        assert len(set(s.tolist())) == len(s) and (np.diff(s.astype(np.int64)) > 0).all()


def test_csr_bitmap_roundtrip():
    rows = datagen.regime_txns(777, 6, 4, 3, 0.3, seed=4)
    rp, it = datagen.txns_to_csr(rows)
    ref, _ = oracle.build_bitmaps(rp, it, 24)
    assert np.array_equal(datagen.csr_to_bitmaps(rp, it, 24), ref)


# ------------------------------------------------------------------ sharding (N>1 bench path)
def _shard_worker(rank, world, port, result_path):
    """One rank of bench.py's N-GPU path with the oracle counting in place of the
    GPU kernel: the same transaction split (txn_shard, row_slice) and the same
    int32 sum all-reduce (allreduce_counts) over gloo."""
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from sgfim import sharding
    n_words = 16 * 7 + 6                      # 7 whole chunks and a ragged end
    bm = datagen.correlated_bitmaps(n_words * 64, 40, 4, 0.05, 0.3, seed=3)
    cp, ci = datagen.walk_candidates(1001, 40, 1, 10, seed=4)
    w0, w1 = sharding.txn_shard(n_words, rank, world)
    part = oracle.support_batch(sharding.row_slice(bm, w0, w1), cp, ci, n_threads=1)
    counts = torch.from_numpy(part.astype(np.int32))
    sharding.allreduce_counts(counts, dist)
    if rank == 0:
        ref = oracle.support_batch(bm, cp, ci, n_threads=1)
        np.save(result_path, np.array([int(np.array_equal(counts.numpy().astype(np.uint32), ref)), len(ref),
                                       w1 - w0]))
    dist.destroy_process_group()


def test_two_rank_transaction_split_supports_gloo(tmp_path):
    import socket
    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    out = str(tmp_path / "r.npy")
    mp.start_processes(_shard_worker, args=(2, port, out), nprocs=2, start_method="spawn")
    ok, n, width0 = np.load(out)
    assert ok == 1 and n == 1001 and width0 % 16 == 0


def test_txn_shard_covers_words_on_chunk_boundaries():
    from sgfim import sharding
    for n_words in (1, 15, 16, 17, 16 * 1024, 31_250):
        for world in (1, 2, 3, 8):
            cuts = [sharding.txn_shard(n_words, r, world) for r in range(world)]
            assert cuts[0][0] == 0 and cuts[-1][1] == n_words
            for (a0, a1), (b0, _) in zip(cuts, cuts[1:]):
                assert a1 == b0 and a0 <= a1 and a0 % 16 == 0
    bm = np.arange(3 * 37, dtype=np.uint64).reshape(3, 37)
    sl = sharding.row_slice(bm, 16, 37)
    assert sl.shape == (3, 22) and np.array_equal(sl[:, :21], bm[:, 16:]) and not sl[:, 21].any()


def test_numpy_lut_counting_equals_oracle():
    from oracle import numpy_lut
    bm = datagen.correlated_bitmaps(64 * 40, 30, 4, 0.05, 0.4, seed=9)
    cp, ci = datagen.walk_candidates(300, 30, 1, 8, seed=10)
    assert np.array_equal(numpy_lut.supports(bm, cp, ci), oracle.support_batch(bm, cp, ci))


def test_masks_to_sets():
    from sgfim.service import masks_to_sets
    m = np.zeros((4, 2), np.uint64)
    m[0, 0] = 0b1011
    m[1, 1] = 1 << 63
    m[2] = [1 << 63, 1]
    assert masks_to_sets(m) == [(0, 1, 3), (127,), (63, 64), ()]
    assert masks_to_sets(np.zeros((0, 2), np.uint64)) == []


def test_label_dataset_appends_one_label_per_row():
    from sgfim.patterns import label_dataset
    rows = [[0, 2], [], [1], [0, 1, 2]]
    rp, it, a, n = label_dataset(rows, [1, 0, 0, 1])
    assert (a, n) == (3, 4)
    got = [list(it[int(rp[r]):int(rp[r + 1])]) for r in range(4)]
    assert got == [[0, 2, 3], [4], [1, 4], [0, 1, 2, 3]]
