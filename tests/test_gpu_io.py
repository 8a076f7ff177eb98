"""File I/O of the context: the lshkit loader that streams a file into device
memory through pinned staging buffers, and the NSG writer that runs on a host
thread (kcna_io.cu)."""
import os

import numpy as np
import pytest

from fastkcna_gb300 import index_io, kcna, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,d", [(3000, 128), (1_000_000, 37)])
def test_upload_lshkit_equals_host_upload(tmp_path, n, d):
    """Rows from the file (at 1M x 37, padded to 40 on the device: three 64 MiB
    chunks, so a staging buffer is reused after its event) give the same exact
    k-NN as the same rows uploaded from host memory."""
    X = np.random.default_rng(n).normal(size=(n, d)).astype(np.float32)
    path = str(tmp_path / "x.lshkit")
    synth.write_lshkit(path, X)
    with open(path, "ab") as f:
        f.write(b"\0\0\0")  # a partial trailing row is ignored, as Matrix::load does
    ids = np.arange(0, n, max(1, n // 97), dtype=np.uint32)
    with kcna.Index(0) as a, kcna.Index(0) as b:
        a.upload(X)
        b.upload_lshkit(path)
        assert b.n == n and b.d == d
        ai, ad = a.knn_exact(ids, 20)
        bi, bd = b.knn_exact(ids, 20)
    assert np.array_equal(ai, bi) and np.array_equal(ad, bd)


def test_upload_lshkit_errors(tmp_path):
    with kcna.Index(0) as ix:
        with pytest.raises(IOError):
            ix.upload_lshkit(str(tmp_path / "missing.lshkit"))
        bad = tmp_path / "bad.lshkit"
        bad.write_bytes(np.array([8, 10, 4], np.uint32).tobytes() + bytes(320))  # element size 8: not float
        with pytest.raises(IOError):
            ix.upload_lshkit(str(bad))


def test_write_nsg_async_equals_sync(tmp_path):
    X = synth.base("c1", 5000)
    kw = dict(K=40, L=40, S=10, R=40, iterations=5, search_L=30, nsg_R=20, search_K=40, controls=20)
    with kcna.Index(0) as ix:
        ix.upload(X)
        ix.build("nsg", kcna.params(**kw))
        ix.write_nsg(str(tmp_path / "sync.nsg"))
        ix.write_nsg_async(str(tmp_path / "async.nsg"))
        g, deg, ep = ix.graph()  # the context stays usable while the file is written
        ix.wait_writes()
        ix.write_nsg_async(str(tmp_path / "nodir" / "x.nsg"))
        with pytest.raises(IOError):
            ix.wait_writes()
    a = (tmp_path / "sync.nsg").read_bytes()
    assert a == (tmp_path / "async.nsg").read_bytes()
    rows, ep2, width = index_io.read_nsg(str(tmp_path / "async.nsg"))
    assert ep2 == ep and [len(r) for r in rows] == deg.tolist()
