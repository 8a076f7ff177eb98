"""CPU-only tests: the C ABI exports, pool-insert semantics, the dataset
generator, the live reference pins (where the reference compiled here) and the
bench's host logic (reference arm, two-rank gloo)."""
import json
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import oracle_py
from conftest import ROOT
from fastkcna_gb300 import synth


def test_abi_exports_every_declared_function():
    import ctypes

    lib_path = os.path.join(ROOT, "fastkcna_gb300", "libkcna.so")
    if not os.path.exists(lib_path):
        from fastkcna_gb300 import build

        build.build()
    lib = ctypes.CDLL(lib_path)  # loads without a GPU; nothing is called
    header = open(os.path.join(ROOT, "include", "kcna.h")).read()
    header = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    names = sorted(set(re.findall(r"\b(kcna_\w+)\s*\(", header)))
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_structs_match_the_c_layout(tmp_path):
    """kcna_params / kcna_stats as the C compiler lays them out, against the
    ctypes mirrors of the product binding and of the oracle binding (a stats
    struct shorter than the C one is overrun by the library's memset)."""
    import ctypes

    from fastkcna_gb300 import kcna

    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "kcna.h"\n'
        "int main(void) {\n"
        '  printf("%zu %zu %zu %zu\\n", sizeof(kcna_params), sizeof(kcna_stats),\n'
        "         offsetof(kcna_stats, prune_tc), offsetof(kcna_stats, prune_skipped));\n"
        "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    p_size, s_size, off_tc, off_skip = map(int, subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.split())
    for Params, Stats in ((kcna.Params, kcna.Stats), (oracle_py.Params, oracle_py.Stats)):
        assert ctypes.sizeof(Params) == p_size
        assert ctypes.sizeof(Stats) == s_size
        assert Stats.prune_tc.offset == off_tc and Stats.prune_skipped.offset == off_skip


def _model_pool(L, cap, entries):
    """Top-`cap` by (distance, insertion order) of unique ids: what the
    sequential try-insert keeps when no distance ties at the boundary."""
    best = {}
    for i, (idx, d) in enumerate(entries):
        if idx not in best:
            best[idx] = (d, i)
    order = sorted(best.items(), key=lambda kv: kv[1])
    return [k for k, _ in order[:cap]]


@pytest.mark.parametrize("seed", range(5))
def test_pool_insert_matches_top_l_model(oracle, seed):
    rng = np.random.default_rng(seed)
    cap = 32
    ids0 = rng.choice(10_000, 10, replace=False).astype(np.uint32)
    d0 = np.sort(rng.random(10).astype(np.float32))
    cid = rng.integers(0, 10_000, 400).astype(np.uint32)
    cd = rng.random(400).astype(np.float32)
    # same id always has the same distance (the distance of a pair is a function of the pair)
    dist_of = {int(i): float(d) for i, d in zip(ids0, d0)}
    for j in range(cid.size):
        cd[j] = dist_of.setdefault(int(cid[j]), float(cd[j]))
    ids, dists, flags, L, rad, ret = oracle.pool_insert_seq(ids0, d0, np.zeros(10, np.uint8), 10, cap, np.inf,
                                                            cid, cd)
    assert L == cap and np.all(np.diff(dists) >= 0) and len(set(ids.tolist())) == L
    model = _model_pool(L, cap, list(zip(ids0.tolist(), d0.tolist())) + list(zip(cid.tolist(), cd.tolist())))
    assert ids.tolist() == model
    assert rad == dists[-1]


def test_synth_shapes_and_ranges():
    x = synth.base("c2", 4096)
    assert x.shape == (4096, 128) and x.dtype == np.float32
    assert x.min() >= 0 and x.max() <= 255 and np.all(x == np.rint(x))
    y = synth.base("c3", 1000)
    np.testing.assert_allclose(np.linalg.norm(y, axis=1), 1.0, rtol=1e-5)
    z = synth.base("c4", 100)
    assert z.shape == (100, 960) and z.min() >= 0
    assert np.array_equal(synth.base("c1", 500), synth.base("c1", 500))


def test_lshkit_round_trip(tmp_path):
    x = synth.base("c1", 300)
    p = str(tmp_path / "x.lshkit")
    synth.write_lshkit(p, x)
    assert np.array_equal(synth.read_lshkit(p), x)
    raw = np.fromfile(p, dtype=np.uint32, count=3)
    assert raw.tolist() == [4, 300, 32]


needs_ref = pytest.mark.skipif(not oracle_py.Reference.available(), reason="reference not compiled here")


@needs_ref
@pytest.mark.parametrize("name", ["c1", "c2"])
def test_oracle_matches_live_reference(oracle, name):
    ref = oracle_py.Reference()
    X = synth.base(name, 3000)
    p = oracle_py.params(K=64, L=64, S=10, R=64, iterations=4, search_L=32, nsg_R=24, search_K=64,
                         tau=0.05 if name == "c1" else 10.0, controls=20)
    ids = np.arange(0, 3000, 101, dtype=np.uint32)
    oi, od = oracle.knn(X, ids, 64)
    ri, rd = ref.linear_search(X, ids, 64)
    assert np.array_equal(oi, ri)
    pid, pd, pc, rec, fin = ref.nndescent(X, p, nthreads=2)
    for kind in (1, 3, 4):
        a = oracle.prune(kind, X, p, pid, pd, pc, 40)
        b = ref.prune(kind, X, p, pid, pd, pc, 40)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2])


@needs_ref
def test_oracle_nndescent_recall_tracks_reference(oracle):
    ref = oracle_py.Reference()
    X = synth.base("c1", 8000)
    p = oracle_py.params(K=64, L=64, S=10, R=64, iterations=6, search_L=32, nsg_R=24, search_K=64, controls=100)
    _, _, _, rec, fin = ref.nndescent(X, p, nthreads=4)
    _, _, _, st = oracle.nndescent(X, p, nthreads=4)
    assert abs(st.loop_recall[0] - fin) < 0.02, (st.loop_recall[0], fin)


def test_bench_reference_arm_prints_one_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "3",
                        "--warmup", "0", "--n", "3000", "--ref-budget", "0"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["unit"] == "s" and j["higher_is_better"] is False
    assert j["cpu_baseline"]["kind"] in ("reference", "port") and j["e2e"]["h2d_bytes_per_step"] == 0
    # whole builds of the named size, as many as the budget allows (here one): no extrapolation
    assert j["steps"] == 1 == len(j["results"]["build_seconds"]) and j["config"]["n"] == 3000
    assert j["value"] == j["cpu_baseline"]["value"] == j["e2e"]["value"]
    import bench

    assert j["config"] == bench.static_config(3000)  # the GPU arm prints the same config


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    ws, r, _ = bench.dist_setup()
    bench.barrier(ws)
    q.put((r, bench.max_over_ranks(ws, float(10 + r))))


def test_bench_two_rank_gloo_max_over_ranks():
    import multiprocessing as mp
    import socket

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    got = sorted(q.get(timeout=5) for _ in ps)
    assert got == [(0, 11.0), (1, 11.0)]


def test_bench_roofline_picks_dominant_phase_and_counts_bf16_bytes():
    import bench

    st = {"phase_ms": {"join": 300.0, "merge": 100.0, "prune": 200.0}, "phase_launches": {"join": 6, "merge": 10, "prune": 3},
          "bf16_rows": 1, "gram_tc": 1, "join_rows": 6_000_000, "cand_emitted": 1_000_000, "cand_merged": 2_000_000,
          "pool_entries_merged": 500_000, "maxl": 500, "loops": 3, "prune_skipped": 0}
    name, r = bench.roofline(st, 6782.4, 128, 1000, 500)
    assert name == "join" and r["kernel"] == "join_tc_kernel" and r["launches_per_step"] == 6
    per_launch = (6_000_000 * 128 * 2 + 1_000_000 * 12) / 6
    assert r["achieved"] == pytest.approx(per_launch / (0.3 / 6) / 1e9, abs=0.06)  # rounded to 0.1 GB/s
    assert r["frac"] == pytest.approx(r["achieved"] / 6782.4, abs=1e-4)
    st["phase_ms"]["prune"] = 400.0
    st["bf16_rows"] = 0
    name, r = bench.roofline(st, 6782.4, 128, 1000, 500)
    assert name == "prune" and r["kernel"] == "prune_kernel"
    assert r["achieved"] == pytest.approx((3 * 1000 * 500 * 128 * 4 / 3) / (0.4 / 3) / 1e9, abs=0.06)
    assert set(r["roofs"]) == {"hbm"}
    # incremental prunes: only the node prunes that ran count
    st["prune_skipped"] = 1200
    name, r = bench.roofline(st, 6782.4, 128, 1000, 500)
    assert r["achieved"] == pytest.approx((1800 * 500 * 128 * 4 / 3) / (0.4 / 3) / 1e9, abs=0.06)


def test_bench_roofline_gram_prune_against_both_roofs():
    import bench

    # C2 1M, learned + BF16: prune 185 ms over 3 launches
    st = {"phase_ms": {"join": 150.0, "merge": 180.0, "prune": 185.0},
          "phase_launches": {"join": 6, "merge": 25, "prune": 3},
          "bf16_rows": 1, "gram_tc": 1, "prune_tc": 1, "join_rows": 1, "cand_emitted": 1, "cand_merged": 1,
          "pool_entries_merged": 1, "maxl": 500, "loops": 3, "prune_skipped": 0}
    name, r = bench.roofline(st, 6774.6, 128, 1_000_000, 500, tensor_tflops=1713.4)
    assert name == "prune" and r["kernel"] == "prune_gram_kernel"
    t = r["roofs"]["tensor"]
    pairs = 500 * 499 // 2
    assert t["achieved"] == pytest.approx(1_000_000 * pairs * 2 * 128 / (0.185 / 3) / 1e12, abs=0.06)
    h = r["roofs"]["hbm"]
    assert h["achieved"] == pytest.approx(1_000_000 * 500 * 128 * 2 / (0.185 / 3) / 1e9, abs=0.06)
    # 128 GB at 6.77 TB/s (18.9 ms) outlasts 31.9 TFLOP at 1.71 PFLOP/s (18.6 ms): HBM is the binding roof
    assert r["bound"] == "hbm" and r["frac"] == h["frac"]
    # at a lower tensor peak the tensor roof binds and becomes the headline
    name, r = bench.roofline(st, 6774.6, 128, 1_000_000, 500, tensor_tflops=1000.0)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s" and r["frac"] == r["roofs"]["tensor"]["frac"]
    # the FP32 prune has no tensor roof
    st["prune_tc"] = 0
    name, r = bench.roofline(st, 6774.6, 128, 1_000_000, 500, tensor_tflops=1713.4)
    assert set(r["roofs"]) == {"hbm"} and r["kernel"] == "prune_kernel"


C_CALLER = r"""
/* A plain C caller of the drop-in boundary: what a cgo/FFI stub would declare. */
#include <stdio.h>
#include "kcna.h"

int build_index(const char *lshkit_path, const char *nsg_path) {
    kcna_ctx *ctx = NULL;
    kcna_params p;
    kcna_stats st;
    uint64_t comps = 0;
    if (kcna_create(&ctx, 0) != KCNA_OK) return 1;
    kcna_params_default(&p);
    p.K = 500; p.L = 500; p.S = 12; p.R = 100; p.iterations = 6;
    p.search_L = 80; p.nsg_R = 50; p.search_K = 500;
    p.learned_seed = 1; p.screen = KCNA_SCREEN_BF16; p.refine = KCNA_REFINE_BRIDGE_VIEW;
    if (kcna_upload_lshkit(ctx, lshkit_path) != KCNA_OK || kcna_build(ctx, &p, KCNA_NSG, &st) != KCNA_OK) {
        fprintf(stderr, "%s\n", kcna_last_error(ctx));
        kcna_destroy(ctx);
        return 2;
    }
    kcna_write_nsg_async(ctx, nsg_path);
    kcna_pool_search(ctx, &p, 1, &comps);
    kcna_prune(ctx, &p, KCNA_CAGRA);
    int rc = kcna_wait_writes(ctx) == KCNA_OK ? 0 : 3;
    kcna_destroy(ctx);
    return rc;
}
"""


def test_c_caller_compiles_and_links(tmp_path):
    """include/kcna.h is plain C: a C99 caller compiles and links against the
    library (not run: no GPU here)."""
    import shutil

    from fastkcna_gb300 import build as kbuild

    if not shutil.which("gcc") or not os.path.exists(kbuild.LIB):
        pytest.skip("gcc or the built library is missing")
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER + "\nint main(int argc, char **argv) { return argc > 2 ? build_index(argv[1], argv[2]) : 0; }\n")
    cuda_lib = "/usr/local/cuda/lib64"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(kbuild.ROOT, "include"), str(src),
                        "-o", str(tmp_path / "caller"), "-L", kbuild.HERE, "-lkcna", "-L", cuda_lib, "-lcudart",
                        f"-Wl,-rpath,{kbuild.HERE}"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
