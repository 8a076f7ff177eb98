"""The fvecs -> lshkit converter (bin/fvec2lshkit, host code only) against
the reference's own src/fvec2lshit.cpp compiled from its sources
(oracle/_ref/fvec2lshit): same output bytes and console lines, and a file the
lshkit readers load back."""
import os
import subprocess

import numpy as np
import pytest

from fastkcna_gb300 import build as kbuild
from fastkcna_gb300 import synth

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "fvec2lshit")


def _tool():
    path = os.path.join(kbuild.BIN, "fvec2lshkit")
    if not os.path.exists(path):
        pytest.skip("converter not built (run __graft_entry__.build())")
    return path


def _write_fvecs(path, x, tail=b""):
    x = np.ascontiguousarray(x, dtype=np.float32)
    rec = np.empty((x.shape[0], x.shape[1] + 1), dtype=np.float32)
    rec[:, 0] = np.frombuffer(np.int32(x.shape[1]).tobytes(), dtype=np.float32)[0]
    rec[:, 1:] = x
    with open(path, "wb") as f:
        f.write(rec.tobytes())
        f.write(tail)


@pytest.mark.parametrize("n,d", [(1000, 17), (1, 128), (3, 960)])
def test_converter_matches_reference(tmp_path, n, d):
    x = np.random.default_rng(n + d).normal(size=(n, d)).astype(np.float32)
    src = tmp_path / "in.fvecs"
    _write_fvecs(src, x, tail=b"\x01\x02\x03")  # a trailing partial record is ignored
    mine = subprocess.run([_tool(), str(src), str(tmp_path / "mine.lshkit")], capture_output=True, text=True,
                          timeout=60)
    assert mine.returncode == 0, mine.stderr
    got = (tmp_path / "mine.lshkit").read_bytes()
    assert got[:12] == np.array([4, n, d], dtype=np.uint32).tobytes()
    assert np.array_equal(synth.read_lshkit(str(tmp_path / "mine.lshkit")), x)
    if not os.path.exists(REF):
        pytest.skip("reference converter not compiled (oracle/build_ref.sh)")
    ref = subprocess.run([REF, str(src), str(tmp_path / "ref.lshkit")], capture_output=True, text=True, timeout=60)
    assert ref.returncode == 0
    assert got == (tmp_path / "ref.lshkit").read_bytes()
    assert mine.stdout == ref.stdout


def test_converter_usage_and_errors(tmp_path):
    r = subprocess.run([_tool()], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "fvec2lshkit <input> <output>"
    # a record whose length field differs: the reference aborts, this tool exits 1
    x = np.ones((4, 8), dtype=np.float32)
    src = tmp_path / "bad.fvecs"
    _write_fvecs(src, x)
    raw = bytearray(src.read_bytes())
    raw[2 * 36: 2 * 36 + 4] = np.int32(7).tobytes()
    src.write_bytes(bytes(raw))
    r = subprocess.run([_tool(), str(src), str(tmp_path / "o.lshkit")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "vector 2 has length 7" in r.stderr
    r = subprocess.run([_tool(), str(tmp_path / "missing.fvecs"), str(tmp_path / "o2.lshkit")], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "cannot open" in r.stderr
