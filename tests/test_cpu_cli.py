"""Host side of the C++ drop-in (no GPU): the command lines' argument parsing
and defaults, the HNSW level assignment against the reference's own
Matrix::getlevel, and the hnswlib file layout of a layered build made by the
reference itself (read back with fastkcna_gb300.index_io)."""
import ctypes as C
import json
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle_py
from fastkcna_gb300 import build as kbuild
from fastkcna_gb300 import index_io, synth

BIN = kbuild.BIN
TOOLS = list(kbuild.TOOLS)


def _tool(name):
    path = os.path.join(BIN, name)
    if not os.path.exists(path):
        pytest.skip("command lines not built (run __graft_entry__.build())")
    return path


def _params(tool, *args):
    r = subprocess.run([_tool(tool), *args, "--print-params"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


@pytest.mark.parametrize("tool", TOOLS)
def test_cli_defaults_are_the_reference_defaults(tool):
    p = _params(tool, "data.lshkit", "out.idx")
    # src/kgraph.h:12-37
    assert (p["K"], p["L"], p["S"], p["R"], p["iterations"], p["controls"], p["seed"]) == (25, 100, 10, 100, 30, 100, 2024)
    assert (p["nsg_R"], p["search_L"], p["search_K"], p["step"], p["massq_S"], p["loop_i"]) == (50, 40, 500, 10, 10, 2)
    assert p["delta"] == pytest.approx(0.002) and p["recall"] == pytest.approx(0.95)
    assert p["tau"] == 0 and p["angle"] == 60 and p["nthreads"] == 40
    assert p["data"] == "data.lshkit" and p["output"] == "out.idx" and p["tool"] == tool


def test_cli_flag_forms():
    p = _params("fastnsg", "--data", "a", "--output=b", "-K", "200", "-L300", "-S", "0", "-R", "64", "-I", "6",
                "--search_L", "80", "--nsg_R", "40", "--search_K", "300", "--massq_S", "12", "--loop_i", "3",
                "--step", "5", "--tau", "10", "--angle", "55.5", "--nt", "16", "--controls", "50", "--seed", "7",
                "--delta", "0.01", "--recall", "0.99", "--result", "r.csv", "--screen", "bf16", "--learned", "1")
    assert p["data"] == "a" and p["output"] == "b" and p["result"] == "r.csv"
    assert p["K"] == 200 and p["L"] == 300 and p["S"] == 200  # -S 0 means S = K (src/fastnsg.cpp:135-137)
    assert (p["R"], p["iterations"], p["search_L"], p["nsg_R"], p["search_K"]) == (64, 6, 80, 40, 300)
    assert (p["massq_S"], p["loop_i"], p["step"], p["nthreads"], p["controls"], p["seed"]) == (12, 3, 5, 16, 50, 7)
    assert p["tau"] == 10 and p["angle"] == pytest.approx(55.5)
    assert p["delta"] == pytest.approx(0.01) and p["recall"] == pytest.approx(0.99)
    assert p["screen"] == 1 and p["learned_seed"] == 1
    assert p["refine"] == 0


def test_cli_refine_flag():
    assert _params("fastnsg", "d.lshkit", "o.nsg", "--refine", "pool")["refine"] == 1
    assert _params("fasttaumng", "d.lshkit", "o.nsg", "--refine=bridge")["refine"] == 0
    r = subprocess.run([_tool("fastnsg"), "d.lshkit", "o.nsg", "--refine", "beam", "--print-params"],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "--refine must be bridge or pool" in r.stderr


def test_cli_usage_and_errors():
    r = subprocess.run([_tool("fasthnsw"), "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "Usage: fasthnsw" in r.stdout and "--nsg_R" in r.stdout
    r = subprocess.run([_tool("fastnsg")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "Usage" in r.stdout  # no data: usage, like the reference
    r = subprocess.run([_tool("fastnsg"), "x", "--bogus"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "unrecognised option" in r.stderr
    r = subprocess.run([_tool("fastnsg"), "x", "-K", "abc"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "bad value" in r.stderr
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "missing.lshkit")
        r = subprocess.run([_tool("fastnsg"), path, os.path.join(td, "o")], capture_output=True, text=True,
                           timeout=60)
        assert r.returncode == 1


def _facade_levels(n, M, seed):
    lib = C.CDLL(kbuild.FACADE)
    d2f = np.empty(n, np.int32)
    pn = np.empty(64, np.int32)
    nl = C.c_uint32(0)
    rc = lib.kgraph_gb300_levels(C.c_uint32(n), C.c_uint32(M), C.c_uint32(seed), d2f.ctypes.data_as(C.c_void_p),
                                 pn.ctypes.data_as(C.c_void_p), C.c_uint32(64), C.byref(nl))
    assert rc == 0
    return d2f, pn[: nl.value]


@pytest.mark.parametrize("n,M,seed", [(1000, 50, 2024), (20000, 16, 1), (100000, 40, 2024)])
def test_hnsw_levels_match_reference(n, M, seed):
    if not os.path.exists(kbuild.FACADE):
        pytest.skip("facade not built")
    if not oracle_py.Reference.available():
        pytest.skip("reference harness not built")
    ref = oracle_py.Reference()
    d2f_r, pn_r = ref.getlevel(n, M, seed)
    d2f, pn = _facade_levels(n, M, seed)
    assert np.array_equal(pn, pn_r)
    assert np.array_equal(d2f, d2f_r)
    assert pn.sum() == n and len(pn) >= 2


def test_reference_hnswlib_file_layout():
    """A layered build by the reference, written in hnswlib layout, read back:
    labels are the level order, every node's levels and list sizes are bounded."""
    if not oracle_py.Reference.available():
        pytest.skip("reference harness not built")
    ref = oracle_py.Reference()
    X = synth.base("c1", 3000)
    p = oracle_py.params(K=40, L=40, S=10, R=40, iterations=4, search_L=20, nsg_R=16, search_K=40, controls=20)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "h.bin")
        ref.build_hnsw(X, p, path, nthreads=4)
        idx = index_io.read_hnswlib(path)
    d2f, pn = ref.getlevel(3000, 16, p.seed)
    assert idx["cur_element_count"] == 3000 and idx["maxM"] == 16 and idx["maxM0"] == 32 and idx["M"] == 16
    assert idx["maxlevel"] == len(pn) - 1
    assert np.array_equal(idx["labels"], d2f.astype(np.uint64))
    assert np.array_equal(idx["data"], X[d2f])
    expect_levels = np.repeat(np.arange(len(pn) - 1, -1, -1), pn[::-1])
    assert np.array_equal(idx["levels"], expect_levels)
    assert max(len(a) for a in idx["level0"]) <= 32
    for l, rows in idx["upper"].items():
        assert all(len(ids) <= 16 and (ids < pn[l:].sum()).all() for _, ids in rows)
    assert idx["levels"][idx["enterpoint"]] == idx["maxlevel"]


def test_hnsw_levels_match_golden_fixture():
    """The level assignment for the command-line test data (20,000 rows,
    nsg_R 32, seed 2024) equals the reference's, as stored in the fixture."""
    if not os.path.exists(kbuild.FACADE):
        pytest.skip("facade not built")
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_cli_c1.npz"))
    d2f, pn = _facade_levels(20000, 32, 2024)
    assert np.array_equal(d2f, g["levels_data2file"]) and np.array_equal(pn, g["levels_points_num"])
