import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    """Golden arrays as a dict of materialised arrays.

    Indexing an NpzFile decompresses a fresh array on every access; a raw
    pointer (``.ctypes.data``) taken from such a temporary dangles as soon as
    the temporary is collected, so tests get held arrays instead.
    """
    cache = {}

    def load(name):
        if name not in cache:
            with np.load(os.path.join(GOLDEN, f"golden_{name}.npz")) as z:
                cache[name] = {k: z[k] for k in z.files}
        return cache[name]
    return load


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def cuda_lib():
    """The CUDA engine; GPU tests fail (not skip) when it cannot load."""
    import das_gb300
    return das_gb300.lib()
