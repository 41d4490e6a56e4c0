"""Reusable permanent plans executed as one CUDA graph.

A :class:`PermanentPlan` plans and uploads a batch of permanents (or Laplace
permanents) of one matrix once; every :meth:`run` is then a single CUDA-graph
launch of the device pipeline — queue reset, persistent walk over a device work
queue, reductions — with no host planning or copies besides reading the
results.  This is the form for repeated batches: the exact probabilities of a
fixed list of output patterns, or benchmark loops.
"""

import ctypes

import numpy as np

from . import _lib
from .permanent import PermanentInputError, _as_matrix, _raise_for


class PermanentPlan:
    def __init__(self, matrix, rows, cols, form="plain", mode="auto"):
        m = _as_matrix(matrix)
        R = np.ascontiguousarray(np.atleast_2d(np.asarray(rows)).astype(np.int32, casting="unsafe"))
        C = np.asarray(cols).astype(np.int32, casting="unsafe")
        if C.ndim == 1:
            C = np.broadcast_to(C, (R.shape[0], C.shape[0]))
        C = np.ascontiguousarray(C)
        if R.shape[1] != m.shape[0] or C.shape != (R.shape[0], m.shape[1]):
            raise PermanentInputError("rows must be (batch, %d) and cols (batch, %d) or (%d,)"
                                      % (m.shape[0], m.shape[1], m.shape[1]))
        self.batch = R.shape[0]
        self.n_cols = m.shape[1]
        self.form = form
        self.single = m.dtype == np.complex64
        self._h = ctypes.c_void_p()
        L = _lib.load()
        st = L.pqg_plan_create(m.ctypes.data_as(ctypes.c_void_p), m.shape[0], m.shape[1],
                               R.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                               C.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), self.batch,
                               1 if self.single else 0, 1 if form == "laplace" else 0, _lib.MODES[mode],
                               ctypes.byref(self._h))
        if st:
            _raise_for(st)

    def launch(self):
        st = _lib.load().pqg_plan_launch(self._h)
        if st:
            _raise_for(st)

    def synchronize(self):
        """Waits for the last launch; returns its device time in ms."""
        ms = ctypes.c_double(0.0)
        st = _lib.load().pqg_plan_synchronize(self._h, ctypes.byref(ms))
        if st:
            _raise_for(st)
        return ms.value

    def read(self):
        per = 1 if self.form == "plain" else max(1, self.n_cols)
        out = np.zeros(2 * per * self.batch, dtype=np.float32 if self.single else np.float64)
        n = ctypes.c_int64(0)
        st = _lib.load().pqg_plan_read(self._h, out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n))
        if st:
            _raise_for(st)
        vals = (out[0::2] + 1j * out[1::2]).astype(np.complex64 if self.single else np.complex128)
        return vals if self.form == "plain" else vals.reshape(self.batch, per)

    def run(self):
        self.launch()
        self.synchronize()
        return self.read()

    def info(self):
        steps = ctypes.c_double(0.0)
        flops = ctypes.c_double(0.0)
        items = ctypes.c_int64(0)
        h2d = ctypes.c_int64(0)
        _lib.load().pqg_plan_info(self._h, ctypes.byref(steps), ctypes.byref(flops), ctypes.byref(items),
                                  ctypes.byref(h2d))
        return {"steps": steps.value, "flops": flops.value, "work_items": items.value, "plan_bytes": h2d.value}

    def close(self):
        if self._h:
            _lib.load().pqg_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
