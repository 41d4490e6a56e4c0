"""CPU tests of the C ABI boundary: the library builds, loads and exports
every symbol include/pqperm_gb300.h declares; input validation happens on the
host before any device work; without a GPU the engine fails loudly."""

import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "pqperm_gb300.h")


def header_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(pqg_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib(engine):
    from piquasso_gb300 import _lib

    return _lib.load()


def test_header_declares_entry_points():
    syms = header_symbols()
    for s in ("pqg_permanent_c128", "pqg_permanent_c64", "pqg_permanent_laplace_c128",
              "pqg_permanent_laplace_c64", "pqg_permanent_batch_c128", "pqg_permanent_batch_c64"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    for s in header_symbols():
        assert hasattr(lib, s), s
        ctypes.cast(getattr(lib, s), ctypes.c_void_p)


def test_python_binding_covers_header():
    from piquasso_gb300 import _lib

    assert sorted(_lib.SIGNATURES) == header_symbols()


def test_version_and_counters(lib):
    assert b"sm_103a" in lib.pqg_version()
    assert lib.pqg_kernel_launches() >= 0


def test_sum_mismatch_rejected_on_host(lib, engine):
    # validated before the device is touched: same answer with or without a GPU
    with pytest.raises(engine.PermanentInputError) as ei:
        engine.permanent(np.eye(2), [1, 1], [2, 1])
    assert isinstance(ei.value, RuntimeError)
    assert "equal" in str(ei.value)
    with pytest.raises(engine.PermanentInputError):
        engine.permanent(np.eye(2), [1, -1], [1, -1])
    with pytest.raises(engine.PermanentTooLarge):
        engine.permanent(np.ones((2, 40)), [20, 20], np.ones(40))
    with pytest.raises(engine.PermanentInputError):
        engine.permanent_batch(np.eye(2), [[1, 1], [2, 1]], [1, 1])


def test_shape_and_dtype_validation(engine):
    with pytest.raises(ValueError):
        engine.permanent(np.eye(2), [1, 1, 1], [1, 1])
    with pytest.raises(TypeError):
        engine.permanent(np.eye(2, dtype=np.clongdouble), [1, 1], [1, 1])
    with pytest.raises(ValueError):
        engine.permanent(np.ones(3), [1], [1])


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a GPU")
def test_no_cpu_fallback_without_gpu(engine):
    with pytest.raises(engine.EngineUnavailable):
        engine.permanent(np.eye(3), [1, 1, 1], [1, 1, 1])
    with pytest.raises(engine.EngineUnavailable):
        engine.permanent_laplace(np.eye(3)[:, :2], [1, 0, 0], [1, 1])


def test_status_codes_match_the_header():
    """Every PQG_ERR_* status of include/pqperm_gb300.h has the same value in
    the Python binding (PQG_ERR_HOST: a host-side failure such as running out
    of host memory, which the entry points return instead of letting a C++
    exception cross the C ABI)."""
    import os
    import re

    from piquasso_gb300 import _lib

    here = os.path.dirname(os.path.abspath(__file__))
    header = open(os.path.join(os.path.dirname(here), "include", "pqperm_gb300.h")).read()
    codes = dict(re.findall(r"#define (PQG_ERR_\w+) (\d+)", header))
    assert "PQG_ERR_HOST" in codes
    for name, value in codes.items():
        assert getattr(_lib, name) == int(value), name
