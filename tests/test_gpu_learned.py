"""Learned seed: encoder gradients against the CPU oracle, and what the trained
encoder gains over the random-start method."""
import ctypes as C

import numpy as np
import pytest

import mlp_oracle
from fastkcna_gb300 import kcna, synth

pytestmark = pytest.mark.gpu


def _grads(index, X, W1, b1, W2, b2, margin):
    lib = kcna.load_library()
    f = lib.kcna_encoder_grads
    f.restype = C.c_int
    P = C.c_void_p
    f.argtypes = [P, P, C.c_uint32, C.c_uint32, P, P, P, P, C.c_float, P, P, P, P, P]
    R, d = X.shape
    loss = np.zeros(1, np.float32)
    dW1 = np.zeros((256, d), np.float32)
    db1 = np.zeros(256, np.float32)
    dW2 = np.zeros((64, 256), np.float32)
    db2 = np.zeros(64, np.float32)
    arrs = [np.ascontiguousarray(a, np.float32) for a in (X, W1, b1, W2, b2)]
    rc = f(index.h, *[a.ctypes.data for a in arrs[:1]], R, d, *[a.ctypes.data for a in arrs[1:]], margin,
           loss.ctypes.data, dW1.ctypes.data, db1.ctypes.data, dW2.ctypes.data, db2.ctypes.data)
    assert rc == 0, rc
    return float(loss[0]), dW1, db1, dW2, db2


def _rel(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.parametrize("d", [32, 128])
def test_encoder_gradients_match_oracle(index, d):
    rng = np.random.default_rng(d)
    B = 96
    X = rng.standard_normal((3 * B, d)).astype(np.float32)
    X[B:2 * B] = X[:B] + 0.3 * rng.standard_normal((B, d)).astype(np.float32)  # positives near anchors
    W1 = (rng.standard_normal((256, d)) / np.sqrt(d)).astype(np.float32)
    b1 = (0.1 * rng.standard_normal(256)).astype(np.float32)
    W2 = (rng.standard_normal((64, 256)) / 16).astype(np.float32)
    b2 = (0.1 * rng.standard_normal(64)).astype(np.float32)
    loss, dW1, db1, dW2, db2 = _grads(index, X, W1, b1, W2, b2, 0.5)
    ol, odW1, odb1, odW2, odb2 = mlp_oracle.encoder_grads(X, W1, b1, W2, b2, 0.5)
    assert abs(loss - ol) <= 1e-3 * max(1.0, abs(ol))
    for g, o in ((dW1, odW1), (db1, odb1), (dW2, odW2), (db2, odb2)):
        assert _rel(g, o) < 1e-2, _rel(g, o)


def test_learned_seed_gains_over_random_start(index):
    """Same data and flags, NN-descent run to the 0.99 recall stop: the learned
    start begins far closer to the KNN graph and stops in fewer iterations than
    the random start, at the same recall bar."""
    X = synth.base("c2", 100_000)
    kw = dict(K=100, L=100, S=12, R=100, iterations=12, search_L=40, nsg_R=32, search_K=100, recall=0.99,
              controls=100)
    index.upload(X)
    plain = index.nndescent(**kw)
    learned = index.nndescent(learned_seed=1, **kw)
    assert learned["seed_loss_last"] < learned["seed_loss_first"]
    assert learned["seed_recall"] > 0.05
    assert learned["iter_recall"][0] > plain["iter_recall"][0] + 0.3, (plain["iter_recall"], learned["iter_recall"])
    assert learned["iterations"] < plain["iterations"], (plain["iter_recall"], learned["iter_recall"])
    assert learned["loop_recall"][0] >= 0.99 and plain["loop_recall"][0] >= 0.99
