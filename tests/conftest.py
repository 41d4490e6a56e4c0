import json
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


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def as_matrix(m):
    a = np.array(m["re"], dtype=np.float64) + 1j * np.array(m["im"], dtype=np.float64)
    if "shape" in m:
        a = a.reshape(m["shape"])
    return a.astype(m["dtype"]) if m["dtype"].startswith("complex") else np.real(a).astype(m["dtype"])


def as_complex(v):
    return complex(v[0], v[1])


def haar_unitary(d, seed):
    """QR of a complex Gaussian with the phase fix: U = Q diag(r_ii / |r_ii|)."""
    rng = np.random.default_rng(seed)
    Z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2)
    Q, R = np.linalg.qr(Z)
    return Q * (np.diag(R) / np.abs(np.diag(R)))


@pytest.fixture(scope="session")
def engine():
    """The built engine on a GPU; builds it if needed."""
    import __graft_entry__

    __graft_entry__.build_engine()
    import piquasso_gb300

    return piquasso_gb300
