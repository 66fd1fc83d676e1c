import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Parity bar for distances and safeties (FP64 path vs the FP64 oracle): 1e-9 mm absolute
# plus 1e-12 relative; infinities and the -1 sentinel must match exactly.
ABS_TOL = 1e-9
REL_TOL = 1e-12
INF = np.finfo(np.float64).max


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def dist_mismatch(gpu, ref, abs_tol=ABS_TOL, rel_tol=REL_TOL):
    """Boolean mask of elements that violate the parity bar."""
    gpu = np.asarray(gpu)
    ref = np.asarray(ref)
    inf_ref = ref == INF
    bad = np.zeros(ref.shape, bool)
    bad |= inf_ref != (gpu == INF)
    fin = ~inf_ref & ~(gpu == INF)
    bad |= fin & (np.abs(gpu - ref) > abs_tol + rel_tol * np.abs(ref))
    return bad


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__
    __graft_entry__.build()
    return torch
