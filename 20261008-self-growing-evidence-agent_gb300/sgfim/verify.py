"""Checks of a mined MFI set that do not go through the miner's search.

For a result of ``Engine.mine`` / ``mine_anytime`` at threshold t on the
handle's dataset:

* supports: every reported support is recounted by the batched support
  kernels;
* antichain: loaded as transactions, each reported set is contained in
  exactly one of them (itself), so no reported set contains another;
* maximality: every single-item extension of every reported set is counted
  (sgfim_frequent_extensions); none may reach t -- the maximality rule of
  mine_mfi (code/pipeline/skab_spike.py:129-135);
* completeness: random greedy maximal walks.  A walk draws a random priority
  for every item and, starting from the empty set, adds the highest-priority
  frequent extension until none is left.  The walk then ends on a maximal
  frequent set, which the result must contain.  (This is the greedy walk
  "add items in a random order while the set stays frequent": an item
  rejected once stays infrequent for every superset.)
"""
from __future__ import annotations

import numpy as np

from .engine import Engine


def _mask_rows(ptr, items, words):
    n = len(ptr) - 1
    out = np.zeros((n, words), np.uint64)
    k = np.diff(ptr).astype(np.int64)
    owner = np.repeat(np.arange(n), k)
    it = items.astype(np.int64)
    np.bitwise_or.at(out, (owner, it >> 6), np.left_shift(np.uint64(1), (it & 63).astype(np.uint64)))
    return out


def _row_bytes(rows):
    return [r.tobytes() for r in rows]


def greedy_walks(eng, thr, n_walks, n_items, seed=0, batch=65536):
    """Maximal frequent sets reached by ``n_walks`` random greedy walks, as uint64
    item masks [n_walks, words]."""
    words = max(1, (n_items + 63) // 64)
    rng = np.random.default_rng(seed)
    found = np.zeros((n_walks, words), np.uint64)
    for w0 in range(0, n_walks, batch):
        nb = min(batch, n_walks - w0)
        prio = rng.random((nb, n_items), dtype=np.float32)
        sets = [[] for _ in range(nb)]
        active = np.arange(nb)
        while len(active):
            ptr = np.zeros(len(active) + 1, np.uint64)
            ptr[1:] = np.cumsum([len(sets[i]) for i in active])
            items = np.array([x for i in active for x in sets[i]], np.uint32)
            ext = eng.frequent_extensions(ptr, items, thr)
            bits = np.unpackbits(ext.view(np.uint8), axis=1, bitorder="little")[:, :n_items].astype(bool)
            has = bits.any(axis=1)
            pick = np.where(bits, prio[active], -1.0).argmax(axis=1)
            for j, i in enumerate(active):
                if has[j]:
                    sets[i].append(int(pick[j]))
            done = active[~has]
            for i in done:
                for x in sets[i]:
                    found[w0 + i, x >> 6] |= np.uint64(1) << np.uint64(x & 63)
            active = active[has]
    return found


def check_mfi_set(eng, res, thr, walks=100_000, seed=0, maximal_batch=1 << 20, engine_factory=Engine):
    """Size-independent checks of ``res`` (a MineResult of ``eng``'s dataset at
    threshold ``thr``).  Returns a dict of booleans and counts.  ``engine_factory``
    opens the second handle of the antichain check."""
    out = {}
    cp, ci, sup = res.ptr.astype(np.uint64), res.items.astype(np.uint32), res.support
    n = len(sup)
    info = eng.info()
    n_items = int(info["n_ids"])
    out["mfis"] = n
    out["supports_recount_equal"] = bool(np.array_equal(eng.support_batch(cp, ci), sup)) if n else True
    out["all_frequent"] = bool((sup >= thr).all())
    if n:
        with engine_factory() as pool:
            pool.load_csr(cp, ci)
            contained = pool.support_batch(cp, ci)
        out["antichain"] = bool((contained == 1).all())
    else:
        out["antichain"] = True
    # every single-item extension of every reported set
    not_maximal = 0
    for s0 in range(0, n, maximal_batch):
        s1 = min(n, s0 + maximal_batch)
        sp = cp[s0:s1 + 1] - cp[s0]
        ext = eng.frequent_extensions(sp, ci[int(cp[s0]):int(cp[s1])], thr)
        not_maximal += int(ext.any(axis=1).sum())
    out["maximal_checked"] = n
    out["not_maximal"] = not_maximal
    out["maximal_all"] = not_maximal == 0
    # completeness: every greedy maximal walk ends on a reported set
    if walks:
        words = max(1, (n_items + 63) // 64)
        have = set(_row_bytes(_mask_rows(cp, ci, words))) if n else set()
        found = greedy_walks(eng, thr, walks, n_items, seed=seed)
        keys = _row_bytes(found)
        missing = sum(1 for k in keys if k not in have)
        out["walks"] = walks
        out["walks_distinct_sets"] = len(set(keys))
        out["walks_missing"] = missing
        out["walks_all_found"] = missing == 0
    return out
