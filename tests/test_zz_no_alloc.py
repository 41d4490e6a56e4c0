"""The allocation-free entry point pqg_permanent_unit_c128_noalloc.

It serves callers that cannot allocate device memory: it reads the matrix from
and writes the result to device memory the caller already owns, and keeps all
intermediate data in the library's fixed device scratch.  This test plays such
a caller: it owns its buffers (allocated here through torch, outside the
library), calls the entry point through the C ABI twice in a row with
different matrices — the scratch keeps the first call's contents, so the
second call also checks that everything that must start at zero is reset —
and compares each result with the regular entry point pqg_permanent_c128
within the complex128 tolerance max(1e-10*|perm|, 1e-14*perm(|A|)).

This file is collected last, so a run that stops at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""

import ctypes

import numpy as np
import pytest

import oracle
from conftest import haar_unitary

pytestmark = pytest.mark.gpu


def _regular(lib, A):
    n = A.shape[0]
    ones = np.ones(n, dtype=np.int32)
    out = np.zeros(2)
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int32)
    st = lib.pqg_permanent_c128(A.ctypes.data_as(dp), n, n, ones.ctypes.data_as(ip), ones.ctypes.data_as(ip),
                                0, out.ctypes.data_as(dp), None)
    assert st == 0, lib.pqg_last_error()
    return complex(out[0], out[1])


def _noalloc(lib, torch, A, stream):
    n = A.shape[0]
    d_matrix = torch.from_numpy(A.view(np.float64).copy()).cuda()  # caller-owned device input
    d_out = torch.zeros(2, dtype=torch.float64, device="cuda")     # caller-owned device output
    torch.cuda.synchronize()
    st = lib.pqg_permanent_unit_c128_noalloc(ctypes.c_void_p(d_matrix.data_ptr()), n,
                                             ctypes.c_void_p(d_out.data_ptr()),
                                             ctypes.c_void_p(stream.cuda_stream))
    assert st == 0, lib.pqg_last_error()
    stream.synchronize()
    return complex(*d_out.cpu().numpy())


def _perm_abs(A):
    """perm(|A|): the double-double oracle up to n = 24, beyond it the
    reference's CPU method (a nonnegative matrix: no cancellation)."""
    n = A.shape[0]
    o = np.ones(n, dtype=int)
    if n <= 24:
        return oracle.perm_abs(A, o, o)
    return float(abs(oracle.port_permanent(np.abs(A).astype(np.complex128), o, o)))


def _check(lib, A, got):
    want = _regular(lib, A)
    tol = max(1e-10 * abs(want), 1e-14 * _perm_abs(A))
    assert abs(got - want) <= tol, (n, got, want, tol)


def test_noalloc_matches_regular_entry_point_twice(engine):
    torch = pytest.importorskip("torch")
    from piquasso_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.current_stream()
    results = []
    for n, seed in ((20, 101), (14, 202)):
        A = haar_unitary(2 * n, seed)[:n, :n].copy()
        got = _noalloc(lib, torch, A, stream)
        _check(lib, A, got)
        results.append(got)
    assert results[0] != results[1]


@pytest.mark.parametrize("n", [1, 2, 32])
def test_noalloc_at_the_documented_bounds(engine, n):
    """n = 1 (no Gray-code digit: the seed alone), n = 2 and n = 32, the
    largest order the fixed scratch takes (2^31 codes)."""
    torch = pytest.importorskip("torch")
    from piquasso_gb300 import _lib

    lib = _lib.load()
    A = haar_unitary(2 * n, 300 + n)[:n, :n].copy()
    got = _noalloc(lib, torch, A, torch.cuda.current_stream())
    if n == 1:
        assert abs(got - A[0, 0]) <= 1e-15 * abs(A[0, 0])
    else:
        _check(lib, A, got)


def test_noalloc_warm_call_allocates_no_device_memory(engine):
    """After a first call on the device, a call leaves the device's free
    memory unchanged (the caller's buffers exist before the measurement)."""
    torch = pytest.importorskip("torch")
    from piquasso_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.current_stream()
    n = 16
    A = haar_unitary(2 * n, 7)[:n, :n].copy()
    d_matrix = torch.from_numpy(A.view(np.float64).copy()).cuda()
    d_out = torch.zeros(2, dtype=torch.float64, device="cuda")
    args = (ctypes.c_void_p(d_matrix.data_ptr()), n, ctypes.c_void_p(d_out.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream))
    assert lib.pqg_permanent_unit_c128_noalloc(*args) == 0, lib.pqg_last_error()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert lib.pqg_permanent_unit_c128_noalloc(*args) == 0, lib.pqg_last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    _check(lib, A, complex(*d_out.cpu().numpy()))


def test_noalloc_rejects_sizes_beyond_the_maximum(engine):
    from piquasso_gb300 import _lib

    lib = _lib.load()
    # rejected before any device work: the pointers are never dereferenced
    st = lib.pqg_permanent_unit_c128_noalloc(ctypes.c_void_p(16), 33, ctypes.c_void_p(16), None)
    assert st == _lib.PQG_ERR_TOO_LARGE
    assert b"PQG_NOALLOC_MAX_N" in lib.pqg_last_error()
