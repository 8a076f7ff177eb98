"""BF16 mode: on data whose values are exactly representable in BF16 the
kernels read a BF16 copy of the rows; distances, and hence prune and link
results, must be bit-identical to the FP32 path.  Float data keeps FP32 rows."""
import numpy as np
import pytest

import oracle_py
from fastkcna_gb300 import kcna, synth

pytestmark = pytest.mark.gpu
KW = dict(K=100, L=100, S=10, R=100, iterations=4, search_L=40, nsg_R=32, search_K=100, tau=10.0, angle=60.0)


@pytest.mark.parametrize("kind", ["nsg", "taumng", "alphapg"])
def test_bf16_rows_prune_link_identical_on_integer_data(index, oracle, kind):
    X = synth.base("c2", 6000)
    pid, pd, pc, _ = oracle.nndescent(X, oracle_py.params(**KW), nthreads=1)
    index.upload(X)
    out = {}
    for screen in (0, 1):
        p = kcna.params(screen=screen, **KW)
        index.set_pools(pid, pd, pc, p)
        index.prune(kind, p)
        g1, d1, _ = index.graph()
        index.set_pools(pid, pd, pc, p)
        index.link(kind, p)
        g2, d2, _ = index.graph()
        out[screen] = (g1, d1, g2, d2)
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_bf16_build_uses_copy_only_when_exact(index):
    kw = dict(K=64, L=64, S=10, R=64, iterations=6, search_L=32, nsg_R=24, search_K=64, controls=50)
    index.upload(synth.base("c2", 20000))
    st = index.build("nsg", screen=1, **kw)
    assert st["bf16_rows"] == 1
    st0 = index.build("nsg", screen=0, **kw)
    assert st0["bf16_rows"] == 0
    assert st["loop_recall"][-1] >= st0["loop_recall"][-1] - 0.01
    index.upload(synth.base("c1", 20000))  # float data: not exact in BF16
    st = index.build("nsg", screen=1, **kw)
    assert st["bf16_rows"] == 0 and st["gram_tc"] == 2  # screened on a rounded copy, rescored in FP32
