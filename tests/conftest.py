import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "spai-gmres-ir_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libspai_ir.so)")


@pytest.fixture(scope="session")
def built():
    """Build the library, CLIs and oracle once per session (nvcc cross-compiles without a GPU)."""
    import __graft_entry__ as g

    g.build()
    return True


GOLDEN = os.path.join(ROOT, "tests", "golden")


def golden(name):
    import numpy as np

    return np.load(os.path.join(GOLDEN, name + ".npz"))


def golden_system(g):
    return (int(g["n"]), g["a_ptr"], g["a_idx"], g["a_val"])
