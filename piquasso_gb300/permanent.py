"""Drop-in replacements for the reference module ``piquasso._math.permanent``.

``permanent(matrix, rows, cols)`` and ``permanent_laplace(matrix, rows, cols)``
keep the reference's names, keyword names, dtype rules, return types and error
behaviour (piquasso/_math/permanent.cpp:26-85 and src/permanent.cpp,
src/permanent_laplace.cpp of the reference), and run on the GPU through the C
ABI in include/pqperm_gb300.h:

* dtype: the reference registers a complex64 overload before a complex128 one
  (permanent.cpp:73-84).  An ndarray is accepted by the first overload its
  dtype casts to safely (numpy "safe" casting); a non-ndarray (a list) is
  converted by the first overload, i.e. to complex64.  Nothing else converts:
  a TypeError is raised, as pybind11 does.
* ``rows`` / ``cols`` are force-cast to int32 (``py::array::forcecast``).
* ``permanent`` returns a 0-d array of the matrix's complex dtype;
  ``permanent_laplace`` a 1-D array of ``len(cols)`` entries, or ``[1]`` for an
  empty input (permanent_laplace.cpp:52-57).
* sum(rows) != sum(cols) raises :class:`PermanentInputError`, which is both a
  ``ValueError`` and a ``RuntimeError`` (the reference surfaces a RuntimeError).

Unlike the reference, ``len(rows)`` and ``len(cols)`` are checked against the
matrix shape (the reference reads out of bounds there).
"""

import ctypes

import numpy as np

from . import _lib


class PermanentInputError(ValueError, RuntimeError):
    """Invalid permanent input (for example sum(rows) != sum(cols))."""


class PermanentTooLarge(ValueError):
    """Beyond the engine's limits (> 32 distinct columns, > 2^50 steps)."""


def _raise_for(status):
    msg = _lib.last_error()
    if status == _lib.PQG_ERR_SUM_MISMATCH:
        raise PermanentInputError(msg or "Number of input and output states should be equal")
    if status == _lib.PQG_ERR_INVALID:
        raise PermanentInputError(msg)
    if status == _lib.PQG_ERR_TOO_LARGE:
        raise PermanentTooLarge(msg)
    if status == _lib.PQG_ERR_NO_DEVICE:
        raise _lib.EngineUnavailable(msg or "no CUDA device visible")
    if status == _lib.PQG_ERR_HOST:
        raise MemoryError(msg)
    raise RuntimeError("piquasso_gb300 engine error %d: %s" % (status, msg))


def _as_matrix(matrix):
    """pybind11's overload resolution for array_t<complex<float>> then <double>."""
    if isinstance(matrix, np.ndarray):
        dt = matrix.dtype
        if np.can_cast(dt, np.complex64, casting="safe"):
            target = np.complex64
        elif np.can_cast(dt, np.complex128, casting="safe"):
            target = np.complex128
        else:
            raise TypeError(
                "permanent(): incompatible function arguments (matrix of dtype %s)" % dt)
        m = np.ascontiguousarray(matrix, dtype=target)
    else:
        try:
            m = np.ascontiguousarray(np.asarray(matrix, dtype=np.complex64))
        except (TypeError, ValueError):
            m = np.ascontiguousarray(np.asarray(matrix, dtype=np.complex128))
    if m.ndim != 2:
        raise PermanentInputError("matrix must be two-dimensional, got shape %s" % (m.shape,))
    return m


def _as_mult(v, n, what):
    a = np.asarray(v)
    if a.size == 0:
        a = np.zeros(0, dtype=np.int32)
    a = np.ascontiguousarray(a.astype(np.int32, casting="unsafe").reshape(-1))
    if a.shape[0] != n:
        raise PermanentInputError("len(%s) = %d does not match the matrix (%d)" % (what, a.shape[0], n))
    return a


def _ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def permanent(matrix, rows, cols):
    """Permanent of ``matrix`` with row multiplicities ``rows`` and column
    multiplicities ``cols`` (BB/FG-Glynn over an n-ary Gray code, Eq. (8) of
    arXiv:2309.07027), computed on the GPU."""
    m = _as_matrix(matrix)
    r = _as_mult(rows, m.shape[0], "rows")
    c = _as_mult(cols, m.shape[1], "cols")
    L = _lib.load()
    if m.dtype == np.complex64:
        out = np.zeros(2, dtype=np.float32)
        st = L.pqg_permanent_c64(_ptr(m, ctypes.c_float), m.shape[0], m.shape[1],
                                 _ptr(r, ctypes.c_int32), _ptr(c, ctypes.c_int32),
                                 _ptr(out, ctypes.c_float))
        if st:
            _raise_for(st)
        return np.array(complex(out[0], out[1]), dtype=np.complex64)
    out = np.zeros(2, dtype=np.float64)
    st = L.pqg_permanent_c128(_ptr(m, ctypes.c_double), m.shape[0], m.shape[1],
                              _ptr(r, ctypes.c_int32), _ptr(c, ctypes.c_int32),
                              _lib.MODE_AUTO, _ptr(out, ctypes.c_double), None)
    if st:
        _raise_for(st)
    return np.array(complex(out[0], out[1]), dtype=np.complex128)


def permanent_dd(matrix, rows, cols, mode="auto"):
    """complex128 permanent with its double-double low words: (value, low).

    ``mode``: "auto" (double-float where valid and the plan is larger than 2^16
    Gray-code steps, else FP64), "fp64" or "df"."""
    m = _as_matrix(np.asarray(matrix, dtype=np.complex128))
    r = _as_mult(rows, m.shape[0], "rows")
    c = _as_mult(cols, m.shape[1], "cols")
    out = np.zeros(2)
    lo = np.zeros(2)
    st = _lib.load().pqg_permanent_c128(
        _ptr(m, ctypes.c_double), m.shape[0], m.shape[1], _ptr(r, ctypes.c_int32),
        _ptr(c, ctypes.c_int32), _lib.MODES[mode], _ptr(out, ctypes.c_double),
        _ptr(lo, ctypes.c_double))
    if st:
        _raise_for(st)
    return complex(out[0], out[1]), complex(lo[0], lo[1])


def permanent_laplace(matrix, rows, cols):
    """For every column l, the permanent with ``cols[l]`` lowered by one
    (Lemma 1 of arXiv:2005.04214), from one Gray-code walk on the GPU."""
    m = _as_matrix(matrix)
    r = _as_mult(rows, m.shape[0], "rows")
    c = _as_mult(cols, m.shape[1], "cols")
    L = _lib.load()
    n = ctypes.c_int64(0)
    single = m.dtype == np.complex64
    ft = np.float32 if single else np.float64
    out = np.zeros(2 * max(1, m.shape[1]), dtype=ft)
    if single:
        st = L.pqg_permanent_laplace_c64(_ptr(m, ctypes.c_float), m.shape[0], m.shape[1],
                                         _ptr(r, ctypes.c_int32), _ptr(c, ctypes.c_int32),
                                         _ptr(out, ctypes.c_float), ctypes.byref(n))
    else:
        st = L.pqg_permanent_laplace_c128(_ptr(m, ctypes.c_double), m.shape[0], m.shape[1],
                                          _ptr(r, ctypes.c_int32), _ptr(c, ctypes.c_int32),
                                          _ptr(out, ctypes.c_double), ctypes.byref(n))
    if st:
        _raise_for(st)
    o = out[: 2 * n.value]
    return (o[0::2] + 1j * o[1::2]).astype(np.complex64 if single else np.complex128)


def permanent_batch(matrix, rows, cols, mode="auto"):
    """Permanents of one matrix for many multiplicity patterns at once.

    ``rows`` has shape (batch, n_rows) and ``cols`` shape (batch, n_cols) (or
    (n_cols,), shared by every pattern).  Returns a (batch,) array of the
    matrix's complex dtype.  One work queue, one walk launch and one
    reduction serve the whole batch.  ``mode`` selects the complex128
    arithmetic ("auto", "fp64" or "df").
    """
    m = _as_matrix(matrix)
    R = np.ascontiguousarray(np.asarray(rows).astype(np.int32, casting="unsafe"))
    if R.ndim != 2 or R.shape[1] != m.shape[0]:
        raise PermanentInputError("rows must have shape (batch, %d)" % m.shape[0])
    batch = R.shape[0]
    C = np.asarray(cols).astype(np.int32, casting="unsafe")
    if C.ndim == 1:
        C = np.broadcast_to(C, (batch, C.shape[0]))
    C = np.ascontiguousarray(C)
    if C.shape != (batch, m.shape[1]):
        raise PermanentInputError("cols must have shape (batch, %d) or (%d,)" % (m.shape[1], m.shape[1]))
    L = _lib.load()
    if m.dtype == np.complex64:
        out = np.zeros(2 * batch, dtype=np.float32)
        st = L.pqg_permanent_batch_c64(_ptr(m, ctypes.c_float), m.shape[0], m.shape[1],
                                       _ptr(R, ctypes.c_int32), _ptr(C, ctypes.c_int32), batch,
                                       _ptr(out, ctypes.c_float))
        cdt = np.complex64
    else:
        out = np.zeros(2 * batch, dtype=np.float64)
        st = L.pqg_permanent_batch_c128(_ptr(m, ctypes.c_double), m.shape[0], m.shape[1],
                                        _ptr(R, ctypes.c_int32), _ptr(C, ctypes.c_int32), batch,
                                        _lib.MODES[mode], _ptr(out, ctypes.c_double))
        cdt = np.complex128
    if st:
        _raise_for(st)
    return (out[0::2] + 1j * out[1::2]).astype(cdt)


def measure_vector_peaks(ms=20.0):
    """Measured FP64 and FP32 FMA throughput of the device, TFLOP/s (2 flops/FMA)."""
    out = np.zeros(2)
    st = _lib.load().pqg_measure_vector_peaks(float(ms), _ptr(out, ctypes.c_double))
    if st:
        _raise_for(st)
    return {"fp64_tflops": float(out[0]), "fp32_tflops": float(out[1])}


def permanent_laplace_batch(matrix, rows, cols):
    """Laplace permanents of one matrix for many multiplicity patterns at once.

    ``rows`` (batch, n_rows), ``cols`` (batch, n_cols).  Returns a
    (batch, n_cols) array; an empty problem (no photons) yields 1 in column 0
    and zeros elsewhere, matching the reference's one-element ``[1]``.
    """
    m = _as_matrix(matrix)
    R = np.ascontiguousarray(np.asarray(rows).astype(np.int32, casting="unsafe"))
    C = np.ascontiguousarray(np.asarray(cols).astype(np.int32, casting="unsafe"))
    if R.ndim != 2 or R.shape[1] != m.shape[0] or C.shape != (R.shape[0], m.shape[1]):
        raise PermanentInputError("rows must be (batch, %d) and cols (batch, %d)" % m.shape)
    batch = R.shape[0]
    nc = max(1, m.shape[1])
    L = _lib.load()
    single = m.dtype == np.complex64
    out = np.zeros(2 * nc * batch, dtype=np.float32 if single else np.float64)
    if single:
        st = L.pqg_permanent_laplace_batch_c64(_ptr(m, ctypes.c_float), m.shape[0], m.shape[1],
                                               _ptr(R, ctypes.c_int32), _ptr(C, ctypes.c_int32), batch,
                                               _ptr(out, ctypes.c_float), None)
    else:
        st = L.pqg_permanent_laplace_batch_c128(_ptr(m, ctypes.c_double), m.shape[0], m.shape[1],
                                                _ptr(R, ctypes.c_int32), _ptr(C, ctypes.c_int32), batch,
                                                _ptr(out, ctypes.c_double), None)
    if st:
        _raise_for(st)
    o = out.reshape(batch, nc, 2)
    return (o[..., 0] + 1j * o[..., 1]).astype(np.complex64 if single else np.complex128)


def sampler_step_batch(matrix, rows, cols, uniforms):
    """One fused step of the batched exact sampler for many shots.

    ``rows`` (batch, d): the output photons each shot has drawn so far (at
    least one); ``cols`` (batch, n_cols): its input photons so far (at least
    one); ``uniforms`` (batch,) in [0, 1).  The Laplace permanents L of every
    shot stay on the GPU, where a second kernel forms the pmf
    p_i = |sum_j cols_j L_j U[i, j]|^2 over the d output modes and draws
    min(#{i : cdf_i < u * cdf_last}, d - 1) — the permanent_laplace call, pmf
    and draw of one iteration of the reference's sampling loop
    (piquasso/_simulators/passive/sampling.py:723-749).  Returns an int64
    array (batch,) of output modes.
    """
    m = _as_matrix(matrix)
    R = np.ascontiguousarray(np.asarray(rows).astype(np.int32, casting="unsafe"))
    C = np.ascontiguousarray(np.asarray(cols).astype(np.int32, casting="unsafe"))
    u = np.ascontiguousarray(np.asarray(uniforms, dtype=np.float64).reshape(-1))
    if R.ndim != 2 or R.shape[1] != m.shape[0] or C.shape != (R.shape[0], m.shape[1]) or len(u) != R.shape[0]:
        raise PermanentInputError("rows must be (batch, %d), cols (batch, %d) and uniforms (batch,)" % m.shape)
    out = np.zeros(R.shape[0], dtype=np.int32)
    L = _lib.load()
    if m.dtype == np.complex64:
        st = L.pqg_sampler_step_c64(_ptr(m, ctypes.c_float), m.shape[0], m.shape[1], _ptr(R, ctypes.c_int32),
                                    _ptr(C, ctypes.c_int32), R.shape[0], _ptr(u, ctypes.c_double),
                                    _ptr(out, ctypes.c_int32))
    else:
        st = L.pqg_sampler_step_c128(_ptr(m, ctypes.c_double), m.shape[0], m.shape[1], _ptr(R, ctypes.c_int32),
                                     _ptr(C, ctypes.c_int32), R.shape[0], _ptr(u, ctypes.c_double),
                                     _ptr(out, ctypes.c_int32))
    if st:
        _raise_for(st)
    return out.astype(np.int64)


def permanent_grad(matrix, rows, cols):
    """Gradient of ``permanent(matrix, rows, cols)`` with respect to every
    matrix entry: G[i, j] = rows[i] * cols[j] * permanent(matrix, rows - e_i,
    cols - e_j), zero where rows[i] or cols[j] is zero — the reference's
    grad_perm (src/permanent.cpp:271-300), i.e. the holomorphic derivative that
    its JAX ``perm`` returns from ``jax.grad(perm, holomorphic=True)``.

    ``matrix`` may carry leading batch dimensions (..., n_rows, n_cols), with
    ``rows`` (..., n_rows) and ``cols`` (..., n_cols) broadcast against them,
    as the reference's PermBwd FFI target (src/jax_perm/jax_perm_core.cpp:
    159-208).  One batched Laplace walk computes every matrix's rows at once.
    Returns an array of the matrix's shape and complex dtype.
    """
    a = np.asarray(matrix)
    if a.ndim < 2:
        raise PermanentInputError("matrix must be at least two-dimensional, got shape %s" % (a.shape,))
    nr, nc = a.shape[-2], a.shape[-1]
    lead = a.shape[:-2]
    batch = int(np.prod(lead)) if lead else 1
    m = _as_matrix(a.reshape(batch * nr, nc)).reshape(batch, nr, nc)
    R = np.ascontiguousarray(np.broadcast_to(np.asarray(rows).astype(np.int32, casting="unsafe"),
                                             lead + (nr,)).reshape(batch, nr))
    C = np.ascontiguousarray(np.broadcast_to(np.asarray(cols).astype(np.int32, casting="unsafe"),
                                             lead + (nc,)).reshape(batch, nc))
    m = np.ascontiguousarray(m)
    L = _lib.load()
    single = m.dtype == np.complex64
    out = np.zeros(2 * batch * nr * nc, dtype=np.float32 if single else np.float64)
    if single:
        st = L.pqg_permanent_grad_c64(_ptr(m, ctypes.c_float), nr, nc, _ptr(R, ctypes.c_int32),
                                      _ptr(C, ctypes.c_int32), batch, _ptr(out, ctypes.c_float))
    else:
        st = L.pqg_permanent_grad_c128(_ptr(m, ctypes.c_double), nr, nc, _ptr(R, ctypes.c_int32),
                                       _ptr(C, ctypes.c_int32), batch, _ptr(out, ctypes.c_double))
    if st:
        _raise_for(st)
    g = (out[0::2] + 1j * out[1::2]).astype(np.complex64 if single else np.complex128)
    return g.reshape(lead + (nr, nc))
