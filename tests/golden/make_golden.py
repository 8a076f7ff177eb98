"""Generates the golden fixtures in this directory from the reference itself.

Runs the reference's own code (oracle/_ref/libkcna_ref.so, compiled from the
reference sources by oracle/build_ref.sh) on two small seeded datasets and
stores its outputs:
  * exact k-NN (LinearSearch, src/kgraph.cpp:309-330) of 40 rows, k = 48;
  * NN-descent pools (KGraphConstructor, src/kgraph.cpp:1281-1459, one thread);
  * sync_prune edge lists of the three kinds on those pools
    (src/kgraph.cpp:1809-1851, 2833-2876, 3157-3203);
  * Link (prune + InterInsert + reversed prune) of the three kinds, one thread
    (src/kgraph.cpp:2087-2143, 3085-3141, 3424-3480);
  * beam search (get_neighbors, src/kgraph.cpp:1560-1623) of 20 queries over
    the NSG link graph from fixed seed ids;
  * into ref_cagra_*.npz, the CAGRA-style rank prune (BuildCagra,
    src/kgraph.cpp:2665-2829) of the stored pools with K = 48 and K = 46, the
    order of equal-rank reverse entries fixed as oracle/ref_harness.cpp states;
  * into ref_pool_search_*.npz, the per-node pool search (inSearch,
    src/kgraph.cpp:2340-2414, 3667-3688) of the stored pools over the stored
    NSG link graph, loops 1 and 2;
  * into ref_refine_*.npz, two P2K refinement steps as buildFastNSG runs them
    between prune loops (src/kgraph.cpp:3813-3843): UpdateNhoods
    (:3537-3584) + BridgeView (:2478-2663) of loop 1 on the stored pools over
    the stored NSG link graph g1, then the NSG link g2 of the refined pools
    and UpdateNhoods + BridgeView of loop 2 over g2 (edges new against g1);
    pools, pool flags, edge flags and distance evaluations of each step;
  * into ref_prune_large_*.npz, sync_prune and Link of the three kinds at the
    C2 flags' sizes (nsg_R = 50, search_K = 500) on 500-entry pools: the
    exact 500-NN lists (LinearSearch) of 2,000 rows, so that the input pools
    are deterministic and need not be stored.
The datasets are stored with the outputs (C2-like rows as uint8).

Usage: python tests/golden/make_golden.py   (needs oracle/_ref built here)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle_py  # noqa: E402
from fastkcna_gb300 import synth  # noqa: E402

N, K, W = 1000, 48, 40
PARAMS = dict(K=K, L=K, S=8, R=48, iterations=5, search_L=24, nsg_R=16, search_K=K, controls=20, massq_S=8,
              angle=60.0)


def make(name, X, tau):
    ref = oracle_py.Reference()
    p = oracle_py.params(**PARAMS, tau=tau)
    out = {"X": X.astype(np.uint8) if name == "c2" else X, "tau": np.float32(tau)}
    ids = np.arange(0, N, 25, dtype=np.uint32)
    out["knn_ids"], out["knn_d"] = ref.linear_search(X, ids, K)
    out["knn_q"] = ids
    pid, pd, pc, rec, fin = ref.nndescent(X, p, nthreads=1)
    out["pool_ids"], out["pool_d"], out["pool_cnt"] = pid, pd, pc
    for kind, tag in ((1, "nsg"), (3, "tau"), (4, "alpha")):
        gi, gd, deg = ref.prune(kind, X, p, pid, pd, pc, W)
        out[f"prune_{tag}_ids"], out[f"prune_{tag}_deg"] = gi, deg
        gi, gd, deg = ref.link(kind, X, p, pid, pd, pc, W)
        out[f"link_{tag}_ids"], out[f"link_{tag}_deg"] = gi, deg
    rng = np.random.default_rng(11)
    Q = synth.queries(name, 20)
    if name == "c2":
        Q = np.rint(Q)
    init = np.stack([rng.choice(N, 24, replace=False) for _ in range(20)]).astype(np.uint32)
    bi, bd = ref.beam_search(X, out["link_nsg_ids"], out["link_nsg_deg"], Q, init, 24, 10)
    out.update(bs_q=Q.astype(np.float32), bs_init=init, bs_ids=bi, bs_d=bd)
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)


def make_cagra(name):
    """CAGRA rank prune of the pools already stored in ref_<name>.npz."""
    ref = oracle_py.Reference()
    z = dict(np.load(os.path.join(HERE, f"ref_{name}.npz")))
    X = z["X"].astype(np.float32)
    out = {}
    for k in (48, 46):
        p = oracle_py.params(**dict(PARAMS, K=k), tau=float(z["tau"]))
        gi, gd, deg = ref.prune(oracle_py.KCNA_CAGRA, X, p, z["pool_ids"], z["pool_d"], z["pool_cnt"], k // 2 + 1)
        out[f"k{k}_ids"], out[f"k{k}_d"], out[f"k{k}_deg"] = gi, gd, deg
    np.savez_compressed(os.path.join(HERE, f"ref_cagra_{name}.npz"), **out)


def make_pool_search(name):
    """inSearch of loops 1 and 2 on the pools and NSG link graph of ref_<name>.npz."""
    ref = oracle_py.Reference()
    z = dict(np.load(os.path.join(HERE, f"ref_{name}.npz")))
    X = z["X"].astype(np.float32)
    p = oracle_py.params(**PARAMS, tau=float(z["tau"]))
    out = {}
    for loop in (1, 2):
        oi, od, oc, scan = ref.pool_search(X, p, z["pool_ids"], z["pool_d"], z["pool_cnt"], z["link_nsg_ids"],
                                           z["link_nsg_deg"], loop, nthreads=1)
        out[f"loop{loop}_ids"], out[f"loop{loop}_d"], out[f"loop{loop}_cnt"] = oi, od, oc
        out[f"loop{loop}_scan"] = np.float32(scan)
    np.savez_compressed(os.path.join(HERE, f"ref_pool_search_{name}.npz"), **out)


def make_refine(name):
    """Two refinement steps (UpdateNhoods + BridgeView, loops 1 and 2) on the
    pools and NSG link graph of ref_<name>.npz, one thread."""
    ref = oracle_py.Reference()
    z = dict(np.load(os.path.join(HERE, f"ref_{name}.npz")))
    X = z["X"].astype(np.float32)
    p = oracle_py.params(**PARAMS, tau=float(z["tau"]), step=8)
    g1, d1 = z["link_nsg_ids"], z["link_nsg_deg"]
    i1, dd1, c1, f1, n1, cc1 = ref.refine(X, p, z["pool_ids"], z["pool_d"], z["pool_cnt"], g1, d1, 1)
    g2, _, d2 = ref.link(1, X, p, i1, dd1, c1, g1.shape[1])
    i2, dd2, c2, f2, n2, cc2 = ref.refine(X, p, i1, dd1, c1, g2, d2, 2, pflags=f1, g_old=g1, g_old_deg=d1)
    out = dict(loop1_ids=i1, loop1_d=dd1, loop1_cnt=c1, loop1_flags=f1, loop1_isnew=n1, loop1_comps=np.uint64(cc1),
               g2_ids=g2, g2_deg=d2, loop2_ids=i2, loop2_d=dd2, loop2_cnt=c2, loop2_flags=f2, loop2_isnew=n2,
               loop2_comps=np.uint64(cc2))
    np.savez_compressed(os.path.join(HERE, f"ref_refine_{name}.npz"), **out)


LARGE_N, LARGE_K, LARGE_W = 2000, 500, 64
LARGE_PARAMS = dict(K=500, L=500, S=12, R=100, iterations=6, search_L=80, nsg_R=50, search_K=500, controls=20,
                    massq_S=10, angle=60.0)


def make_prune_large(name, tau):
    """Prune and Link of the three kinds with nsg_R = 50, search_K = 500 on the
    exact 500-NN pools of 2,000 rows (ids stored as uint16)."""
    ref = oracle_py.Reference()
    X = synth.base(name, LARGE_N)
    if name == "c2":
        X = X.astype(np.uint8).astype(np.float32)
    ids = np.arange(LARGE_N, dtype=np.uint32)
    pid, pd = ref.linear_search(X, ids, LARGE_K)
    pc = np.full(LARGE_N, LARGE_K, np.uint32)
    p = oracle_py.params(**LARGE_PARAMS, tau=tau)
    out = {"X": X.astype(np.uint8) if name == "c2" else X, "tau": np.float32(tau)}
    for kind, tag in ((1, "nsg"), (3, "tau"), (4, "alpha")):
        gi, _, deg = ref.prune(kind, X, p, pid, pd, pc, LARGE_W)
        out[f"prune_{tag}_ids"], out[f"prune_{tag}_deg"] = gi.astype(np.uint16), deg.astype(np.uint16)
        gi, _, deg = ref.link(kind, X, p, pid, pd, pc, 2 * LARGE_W)
        out[f"link_{tag}_ids"], out[f"link_{tag}_deg"] = gi.astype(np.uint16), deg.astype(np.uint16)
    np.savez_compressed(os.path.join(HERE, f"ref_prune_large_{name}.npz"), **out)


if __name__ == "__main__":
    if not oracle_py.Reference.available():
        sys.exit("oracle/_ref/libkcna_ref.so is missing: run oracle/build_ref.sh")
    make("c1", synth.base("c1", N), 0.05)
    make("c2", synth.base("c2", N), 10.0)
    make_cagra("c1")
    make_cagra("c2")
    make_pool_search("c1")
    make_pool_search("c2")
    make_refine("c1")
    make_refine("c2")
    make_prune_large("c1", 0.05)
    make_prune_large("c2", 10.0)
    print("wrote", sorted(f for f in os.listdir(HERE) if f.endswith(".npz")))
