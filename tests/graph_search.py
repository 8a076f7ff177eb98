"""Host searchers used by the tests to score built indexes: a greedy beam
search over an NSG-style graph and the layered HNSW search (greedy descent
through the upper levels, then a beam of width ef on level 0).  Plain NumPy,
squared L2."""
import heapq

import numpy as np


def beam_search(X, adj, entries, q, ef, k):
    """Best-first search from `entries`; adj[i] is an id array."""
    dist = lambda ids: ((X[ids] - q) ** 2).sum(axis=1)
    seen = set(int(e) for e in entries)
    e = np.fromiter(seen, dtype=np.int64)
    de = dist(e)
    cand = [(float(d), int(i)) for d, i in zip(de, e)]
    heapq.heapify(cand)
    best = [(-float(d), int(i)) for d, i in zip(de, e)]  # max-heap of the ef best
    heapq.heapify(best)
    while len(best) > ef:
        heapq.heappop(best)
    while cand:
        d, u = heapq.heappop(cand)
        if len(best) >= ef and d > -best[0][0]:
            break
        nb = [int(v) for v in adj[u] if int(v) not in seen]
        if not nb:
            continue
        seen.update(nb)
        nb = np.asarray(nb, dtype=np.int64)
        for dv, v in zip(dist(nb), nb):
            dv = float(dv)
            if len(best) < ef or dv < -best[0][0]:
                heapq.heappush(cand, (dv, int(v)))
                heapq.heappush(best, (-dv, int(v)))
                if len(best) > ef:
                    heapq.heappop(best)
    out = sorted((-d, i) for d, i in best)
    return np.array([i for _, i in out[:k]], dtype=np.int64)


def seeded_entries(n, ep, count, seed=7):
    """The entry point plus count-1 distinct seeded random nodes: the initial
    pool of the NSG-style searches (the entry point alone does not cross
    between well separated clusters)."""
    rng = np.random.default_rng(seed)
    extra = rng.choice(n, size=min(count, n), replace=False)
    return [int(ep)] + [int(v) for v in extra if int(v) != int(ep)][: count - 1]


def hnsw_search(idx, Q, ef, k, extra_entries=0):
    """Labels of the k nearest found for each query of an index read by
    fastkcna_gb300.index_io.read_hnswlib (extra_entries seeded random nodes
    join the level-0 beam's start)."""
    X = idx["data"]
    upper = {l: dict((i, ids) for i, ids in rows) for l, rows in idx["upper"].items()}
    res = []
    for q in Q:
        cur = int(idx["enterpoint"])
        dcur = float(((X[cur] - q) ** 2).sum())
        for l in range(int(idx["maxlevel"]), 0, -1):
            adj = upper.get(l, {})
            moved = True
            while moved:
                moved = False
                nb = adj.get(cur)
                if nb is None or nb.size == 0:
                    break
                dn = ((X[nb] - q) ** 2).sum(axis=1)
                j = int(np.argmin(dn))
                if dn[j] < dcur:
                    cur, dcur, moved = int(nb[j]), float(dn[j]), True
        start = seeded_entries(X.shape[0], cur, extra_entries + 1) if extra_entries else [cur]
        found = beam_search(X, idx["level0"], start, q, max(ef, k), k)
        res.append(idx["labels"][found].astype(np.int64))
    return np.array(res)
