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


def test_noalloc_matches_regular_entry_point_twice(engine):
    torch = pytest.importorskip("torch")
    from piquasso_gb300 import _lib

    lib = _lib.load()
    stream = torch.cuda.current_stream()
    results = []
    for n, seed in ((20, 101), (14, 202)):
        A = haar_unitary(2 * n, seed)[:n, :n].copy()
        d_matrix = torch.from_numpy(A.view(np.float64).copy()).cuda()  # caller-owned device input
        d_out = torch.zeros(2, dtype=torch.float64, device="cuda")     # caller-owned device output
        torch.cuda.synchronize()
        st = lib.pqg_permanent_unit_c128_noalloc(ctypes.c_void_p(d_matrix.data_ptr()), n,
                                                 ctypes.c_void_p(d_out.data_ptr()),
                                                 ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, lib.pqg_last_error()
        stream.synchronize()
        got = complex(*d_out.cpu().numpy())
        want = _regular(lib, A)
        o = np.ones(n, dtype=int)
        tol = max(1e-10 * abs(want), 1e-14 * oracle.perm_abs(A, o, o))
        assert abs(got - want) <= tol, (n, got, want, tol)
        results.append(got)
    assert results[0] != results[1]


def test_noalloc_rejects_sizes_beyond_the_maximum(engine):
    from piquasso_gb300 import _lib

    lib = _lib.load()
    # rejected before any device work: the pointers are never dereferenced
    st = lib.pqg_permanent_unit_c128_noalloc(ctypes.c_void_p(16), 33, ctypes.c_void_p(16), None)
    assert st == _lib.PQG_ERR_TOO_LARGE
    assert b"PQG_NOALLOC_MAX_N" in lib.pqg_last_error()
