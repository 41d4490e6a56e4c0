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


def test_mlp_entry_points_reject_on_the_host(lib):
    """The MLP GEMM with the transposed output and the one-launch Adam check
    their arguments before any device work (placeholder pointers are never
    read): a non-BF16 epilogue, a transposed row stride below M or not a
    multiple of 8, column sums without a scratch; a tensor count outside
    1..16, a missing tensor."""
    from piquasso_gb300 import _lib

    bad = _lib.PQG_ERR_INVALID
    p = ctypes.c_void_p(256)
    f = ctypes.cast(p, ctypes.POINTER(ctypes.c_float))
    M, N, K = 1024, 256, 256
    args = (p, K, p, K, M, N, K)
    assert lib.pqg_mlp_gemm_tc_t(*args, 0, f, None, None, None, p, M, None, None, None) == bad
    assert lib.pqg_mlp_gemm_tc_t(*args, 1, f, p, f, None, None, M, None, None, None) == bad
    assert lib.pqg_mlp_gemm_tc_t(*args, 1, f, p, f, None, p, M - 8, None, None, None) == bad
    assert lib.pqg_mlp_gemm_tc_t(*args, 4, f, p, None, f, p, M + 4, None, None, None) == bad
    assert lib.pqg_mlp_gemm_tc_t(*args, 4, f, p, None, f, p, M, f, None, None) == bad
    P = ctypes.c_void_p * 2
    R = ctypes.c_int64 * 2
    ptrs = P(256, 512)
    rc = R(4, 4)
    assert lib.pqg_mlp_adam_multi(0, ptrs, None, None, ptrs, ptrs, ptrs, rc, rc, 1e-3, 0.9, 0.999, 1e-8, 1,
                                  None) == bad
    assert lib.pqg_mlp_adam_multi(17, ptrs, None, None, ptrs, ptrs, ptrs, rc, rc, 1e-3, 0.9, 0.999, 1e-8, 1,
                                  None) == bad
    holes = P(256, None)
    assert lib.pqg_mlp_adam_multi(2, holes, None, None, ptrs, ptrs, ptrs, rc, rc, 1e-3, 0.9, 0.999, 1e-8, 1,
                                  None) == bad
    assert lib.pqg_mlp_adam_multi(2, ptrs, None, None, ptrs, ptrs, ptrs, rc, R(4, 0), 1e-3, 0.9, 0.999, 1e-8, 1,
                                  None) == bad
