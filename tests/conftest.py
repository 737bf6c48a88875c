import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    """Golden fixture as (dict of arrays, ColliderSet or None)."""
    from distance3d_gb300.collider_set import ColliderSet
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    cs = None
    if "types" in g:
        cs = ColliderSet(g["types"], g["poses"], g["params"], g["hull_offset"],
                         g["hull_count"], g["vertices"], g.get("links"))
    return g, cs


@pytest.fixture(scope="session")
def golden():
    return load_golden
