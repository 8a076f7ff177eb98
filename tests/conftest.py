import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle():
    import oracle_py

    return oracle_py.Oracle()


@pytest.fixture(scope="session")
def index():
    from fastkcna_gb300 import kcna

    ix = kcna.Index(0)
    yield ix
    ix.close()


def rows_equal_as_sets(a_ids, a_deg, b_ids, b_deg):
    """Count of rows whose edge sets differ."""
    bad = 0
    for i in range(a_ids.shape[0]):
        if set(a_ids[i, : a_deg[i]].tolist()) != set(b_ids[i, : b_deg[i]].tolist()):
            bad += 1
    return bad


def recall_at(found, truth, k):
    hit = 0
    for f, t in zip(found, truth):
        hit += len(set(f[:k].tolist()) & set(t[:k].tolist()))
    return hit / (len(truth) * k)
