"""Oracle for the permanent hot path — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may use this
package, and only as the checker (or the timed CPU baseline).  The product
package ``piquasso_gb300`` never imports it.

Contents:
  * ``permanent_dd`` / ``permanent_laplace_dd``: double-double restatement of
    src/permanent.cpp:49-264 and src/permanent_laplace.cpp:43-240 (reference paths).
  * ``perm_abs``: perm(|A|), the scale in the complex128 tolerance
    max(1e-10*|perm|, 1e-14*perm(|A|)).
  * ``port_permanent`` / ``port_laplace``: the reference's CPU method in its own
    arithmetic and threading (the CPU baseline where the reference module is absent).
  * ``reference_module()``: the reference's own pybind module when it was built
    here by oracle/build_ref.sh (None elsewhere).
  * ``grad_perm``: restatement of the reference's permanent gradient
    (src/permanent.cpp:271-300), minor by minor, over any permanent function.
  * ``sampler``: numpy restatement of the Clifford & Clifford B sampler.
"""

import ctypes
import importlib
import os
import sys

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            _build.build(with_reference=False)
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        fp = ctypes.POINTER(ctypes.c_float)
        ip = ctypes.POINTER(ctypes.c_int)
        for name in ("pqo_permanent_dd", "pqo_permanent_laplace_dd"):
            f = getattr(L, name)
            f.argtypes = [dp, ctypes.c_int, ctypes.c_int, ip, ip, ctypes.c_int, dp]
            f.restype = ctypes.c_int
        for name, p in (
            ("pqo_port_permanent_c128", dp),
            ("pqo_port_laplace_c128", dp),
            ("pqo_port_permanent_c64", fp),
            ("pqo_port_laplace_c64", fp),
        ):
            f = getattr(L, name)
            f.argtypes = [p, ctypes.c_int, ctypes.c_int, ip, ip, ctypes.c_int, p]
            f.restype = ctypes.c_int
        _lib = L
    return _lib


def _prep(matrix, rows, cols, dtype=np.complex128):
    m = np.ascontiguousarray(np.asarray(matrix), dtype=dtype)
    if m.ndim != 2:
        raise ValueError("matrix must be 2-D")
    r = np.ascontiguousarray(np.asarray(rows), dtype=np.int32).reshape(-1)
    c = np.ascontiguousarray(np.asarray(cols), dtype=np.int32).reshape(-1)
    if r.shape[0] != m.shape[0] or c.shape[0] != m.shape[1]:
        raise ValueError("rows/cols lengths must match the matrix shape")
    return m, r, c


def _ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _segments():
    return max(1, 4 * (os.cpu_count() or 1))


def permanent_dd(matrix, rows, cols):
    """Double-double permanent; returns (hi, lo) as two complex128 numbers."""
    m, r, c = _prep(matrix, rows, cols)
    out = np.zeros(4)
    rc = lib().pqo_permanent_dd(
        _ptr(m, ctypes.c_double), m.shape[0], m.shape[1], _ptr(r, ctypes.c_int),
        _ptr(c, ctypes.c_int), _segments(), _ptr(out, ctypes.c_double))
    if rc != 0:
        raise ValueError("Number of input and output states should be equal")
    return complex(out[0], out[1]), complex(out[2], out[3])


def permanent(matrix, rows, cols):
    """Double-double permanent rounded to complex128."""
    hi, lo = permanent_dd(matrix, rows, cols)
    return hi + lo


def perm_abs(matrix, rows, cols):
    """perm(|A|) with the same multiplicities (a nonnegative real number)."""
    m, r, c = _prep(matrix, rows, cols)
    hi, lo = permanent_dd(np.abs(m).astype(np.complex128), r, c)
    return abs((hi + lo).real)


def permanent_laplace_dd(matrix, rows, cols):
    """Double-double Laplace permanents; returns complex128 array (hi + lo)."""
    m, r, c = _prep(matrix, rows, cols)
    out = np.zeros(4 * max(1, m.shape[1]))
    n = lib().pqo_permanent_laplace_dd(
        _ptr(m, ctypes.c_double), m.shape[0], m.shape[1], _ptr(r, ctypes.c_int),
        _ptr(c, ctypes.c_int), _segments(), _ptr(out, ctypes.c_double))
    o = out[: 4 * n].reshape(n, 4)
    return (o[:, 0] + o[:, 2]) + 1j * (o[:, 1] + o[:, 3])


def c128_tolerance(matrix, rows, cols, value=None):
    """max(1e-10*|perm|, 1e-14*perm(|A|)) for complex128 results."""
    if value is None:
        value = permanent(matrix, rows, cols)
    return max(1e-10 * abs(value), 1e-14 * perm_abs(matrix, rows, cols))


def port_permanent(matrix, rows, cols, nthreads=0):
    """The reference CPU method (complex64 or complex128 by the matrix dtype)."""
    mat = np.asarray(matrix)
    single = mat.dtype == np.complex64
    m, r, c = _prep(mat, rows, cols, np.complex64 if single else np.complex128)
    if single:
        out = np.zeros(2, dtype=np.float32)
        rc = lib().pqo_port_permanent_c64(
            _ptr(m, ctypes.c_float), m.shape[0], m.shape[1], _ptr(r, ctypes.c_int),
            _ptr(c, ctypes.c_int), nthreads, _ptr(out, ctypes.c_float))
    else:
        out = np.zeros(2, dtype=np.float64)
        rc = lib().pqo_port_permanent_c128(
            _ptr(m, ctypes.c_double), m.shape[0], m.shape[1], _ptr(r, ctypes.c_int),
            _ptr(c, ctypes.c_int), nthreads, _ptr(out, ctypes.c_double))
    if rc != 0:
        raise ValueError("Number of input and output states should be equal")
    return (out[0] + 1j * out[1]).astype(np.complex64 if single else np.complex128)


def port_laplace(matrix, rows, cols, nthreads=0):
    mat = np.asarray(matrix)
    single = mat.dtype == np.complex64
    m, r, c = _prep(mat, rows, cols, np.complex64 if single else np.complex128)
    ft = np.float32 if single else np.float64
    out = np.zeros(2 * max(1, m.shape[1]), dtype=ft)
    fn = lib().pqo_port_laplace_c64 if single else lib().pqo_port_laplace_c128
    ct = ctypes.c_float if single else ctypes.c_double
    n = fn(_ptr(m, ct), m.shape[0], m.shape[1], _ptr(r, ctypes.c_int), _ptr(c, ctypes.c_int),
           nthreads, _ptr(out, ct))
    o = out[: 2 * n]
    return (o[0::2] + 1j * o[1::2]).astype(np.complex64 if single else np.complex128)


def reference_module():
    """The reference's own ``piquasso._math.permanent`` module, or None."""
    ref_root = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref")
    if not os.path.isdir(os.path.join(ref_root, "piquasso", "_math")):
        return None
    if ref_root not in sys.path:
        sys.path.insert(0, ref_root)
    try:
        return importlib.import_module("piquasso._math.permanent")
    except ImportError:
        return None


def grad_perm(matrix, rows, cols, perm=None):
    """G[i, j] = rows[i] * cols[j] * perm(A; rows - e_i, cols - e_j), zero where
    rows[i] or cols[j] is zero (src/permanent.cpp:271-300: the same loop over
    (i, j), one permanent per minor).  ``perm`` defaults to the double-double
    ``permanent``; pass the reference module's ``permanent`` to follow it
    bit for bit.  Returns an (n_rows, n_cols) complex128 array."""
    A = np.asarray(matrix)
    rows = np.asarray(rows).astype(np.int64)
    cols = np.asarray(cols).astype(np.int64)
    perm = perm or permanent
    G = np.zeros(A.shape, dtype=np.complex128)
    for i in range(A.shape[0]):
        for j in range(A.shape[1]):
            if rows[i] == 0 or cols[j] == 0:
                continue
            r2 = rows.copy()
            r2[i] -= 1
            c2 = cols.copy()
            c2[j] -= 1
            G[i, j] = float(rows[i]) * float(cols[j]) * complex(perm(A, r2, c2))
    return G
