import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "mauve-py_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", name))


def load_mds42():
    """The reference's recoded E. coli fixture pair (ASCII bases), its seed
    and the reference's match list (tests/golden/mds42.npz)."""
    import numpy as np
    g = load_golden("mds42.npz")

    def unpack(p, n):
        v = np.stack([(p >> 6) & 3, (p >> 4) & 3, (p >> 2) & 3, p & 3], axis=1).reshape(-1)[:n]
        return np.frombuffer(b"ACGT", np.uint8)[v]

    return (unpack(g["a"], int(g["na"])), unpack(g["b"], int(g["nb"])), int(g["seed"]), g["matches"])
