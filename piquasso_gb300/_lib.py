"""ctypes binding of the C ABI in include/pqperm_gb300.h.

The library is built in-tree (``piquasso_gb300/build.py``) and loaded from
``piquasso_gb300/_lib/``.  There is no fallback: if it is missing or no CUDA
device is visible, every entry point raises.
"""

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpqperm_gb300.so")

PQG_OK = 0
PQG_ERR_SUM_MISMATCH = 1
PQG_ERR_INVALID = 2
PQG_ERR_TOO_LARGE = 3
PQG_ERR_CUDA = 4
PQG_ERR_NO_DEVICE = 5
PQG_ERR_HOST = 6

MODE_AUTO = 0
MODE_FP64 = 1
MODE_DF = 2
MODES = {"auto": MODE_AUTO, "fp64": MODE_FP64, "df": MODE_DF}

# (name, argtypes) of every symbol the header declares
_d = ctypes.POINTER(ctypes.c_double)
_f = ctypes.POINTER(ctypes.c_float)
_i32 = ctypes.POINTER(ctypes.c_int32)
_i64 = ctypes.POINTER(ctypes.c_int64)
_i8 = ctypes.POINTER(ctypes.c_int8)
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32

SIGNATURES = {
    "pqg_last_error": ([], ctypes.c_char_p),
    "pqg_version": ([], ctypes.c_char_p),
    "pqg_kernel_launches": ([], ctypes.c_uint64),
    "pqg_permanent_c128": ([_d, _I64, _I64, _i32, _i32, _I32, _d, _d], ctypes.c_int),
    "pqg_permanent_c64": ([_f, _I64, _I64, _i32, _i32, _f], ctypes.c_int),
    "pqg_permanent_batch_c128": ([_d, _I64, _I64, _i32, _i32, _I64, _I32, _d], ctypes.c_int),
    "pqg_permanent_batch_c64": ([_f, _I64, _I64, _i32, _i32, _I64, _f], ctypes.c_int),
    "pqg_permanent_laplace_c128": ([_d, _I64, _I64, _i32, _i32, _d, _i64], ctypes.c_int),
    "pqg_permanent_laplace_c64": ([_f, _I64, _I64, _i32, _i32, _f, _i64], ctypes.c_int),
    "pqg_permanent_laplace_batch_c128": ([_d, _I64, _I64, _i32, _i32, _I64, _d, _i64], ctypes.c_int),
    "pqg_permanent_laplace_batch_c64": ([_f, _I64, _I64, _i32, _i32, _I64, _f, _i64], ctypes.c_int),
    "pqg_sampler_step_c128": ([_d, _I64, _I64, _i32, _i32, _I64, _d, _i32], ctypes.c_int),
    "pqg_sampler_step_c64": ([_f, _I64, _I64, _i32, _i32, _I64, _d, _i32], ctypes.c_int),
    "pqg_permanent_grad_c128": ([_d, _I64, _I64, _i32, _i32, _I64, _d], ctypes.c_int),
    "pqg_permanent_grad_c64": ([_f, _I64, _I64, _i32, _i32, _I64, _f], ctypes.c_int),
    "pqg_binomial_moments_c128": ([_d, _I64, _i32, _i32, _I32, _I32, _d, _I64], ctypes.c_int),
    "pqg_plan_create": ([ctypes.c_void_p, _I64, _I64, _i32, _i32, _I64, _I32, _I32, _I32,
                         ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "pqg_plan_launch": ([ctypes.c_void_p], ctypes.c_int),
    "pqg_plan_synchronize": ([ctypes.c_void_p, _d], ctypes.c_int),
    "pqg_plan_read": ([ctypes.c_void_p, ctypes.c_void_p, _i64], ctypes.c_int),
    "pqg_plan_info": ([ctypes.c_void_p, _d, _d, _i64, _i64], ctypes.c_int),
    "pqg_plan_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "pqg_permanent_unit_c128_noalloc": ([ctypes.c_void_p, _I64, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "pqg_mlp_gemm_tc": ([ctypes.c_void_p, _I64, ctypes.c_void_p, _I64, _I64, _I64, _I64, _I32, _f,
                         ctypes.c_void_p, _f, _f, _f, _I32, ctypes.c_void_p], ctypes.c_int),
    "pqg_mlp_gemm_tc_t": ([ctypes.c_void_p, _I64, ctypes.c_void_p, _I64, _I64, _I64, _I64, _I32, _f,
                           ctypes.c_void_p, _f, _f, ctypes.c_void_p, _I64, _f, _f, ctypes.c_void_p], ctypes.c_int),
    "pqg_mlp_transpose_bf16": ([ctypes.c_void_p, _I64, _I64, _I64, ctypes.c_void_p, _I64, ctypes.c_void_p],
                               ctypes.c_int),
    "pqg_mlp_tc_status": ([_i32], ctypes.c_int),
    "pqg_mlp_bias_grad": ([_f, _I64, _I64, _f, _f, ctypes.c_void_p], ctypes.c_int),
    "pqg_mlp_softmax_xent": ([_f, _I64, _I32, _I32, _i8, _i8, _i8, ctypes.c_float, _f, _f, ctypes.c_void_p,
                              ctypes.c_void_p], ctypes.c_int),
    "pqg_mlp_adam": ([_f, ctypes.c_void_p, _f, _f, _f, _I64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                      ctypes.c_float, _I64, ctypes.c_void_p], ctypes.c_int),
    "pqg_mlp_adam_multi": ([_I32] + [ctypes.POINTER(ctypes.c_void_p)] * 6 + [ctypes.POINTER(ctypes.c_int64)] * 2 +
                           [ctypes.c_float] * 4 + [_I64, ctypes.c_void_p], ctypes.c_int),
    "pqg_proposal_features": ([_I32, _I32, _I32, _I32, _f, _i32, _f, ctypes.c_void_p, _i8, _i8, ctypes.c_void_p],
                              ctypes.c_int),
    "pqg_proposal_sample": ([_I32, _I32, _I32, _f, _i8, _i8, ctypes.c_uint64, ctypes.c_void_p, _i8, _i32, _f, _f,
                             _f, _f, ctypes.c_void_p], ctypes.c_int),
    "pqg_proposal_step_tc": ([_I32, _I32, _I32, _I32, _f] + [ctypes.c_void_p] * 4 + [_f] * 4 +
                             [ctypes.c_uint64, ctypes.c_void_p, _i8, _i32, _f, _f, _f, ctypes.c_void_p], ctypes.c_int),
    "pqg_set_tuning": ([_I64, _I64, _I64], ctypes.c_int),
    "pqg_get_tuning": ([_i64, _i64, _i64], ctypes.c_int),
    "pqg_measure_vector_peaks": ([ctypes.c_double, _d], ctypes.c_int),
    "pqg_last_timing": ([_d, _d, _d, _d, _d, _d], ctypes.c_int),
    "pqg_last_walk_kernel": ([_i32, _i32], ctypes.c_int),
    "pqg_set_blocks_per_sm": ([_I32], ctypes.c_int),
    "pqg_tuning_add": ([_I32, _I32, _I32, _I32, ctypes.c_double, ctypes.c_double, _I64, _I64, _I64, _I64, _I64,
                        _I32], ctypes.c_int),
    "pqg_tuning_clear": ([], ctypes.c_int),
    "pqg_tuning_count": ([_i64], ctypes.c_int),
    "pqg_plan_config": ([ctypes.c_void_p, _i64, _i64, _i64, _i32], ctypes.c_int),
    "pqg_device_info": ([ctypes.c_char_p, _I64, _i32], ctypes.c_int),
}

# walk kernel tables (PQG_WALK_* in the header), as pqg_last_walk_kernel reports them
WALK_TABLES = {
    0: "plain_fp64", 1: "plain_c64", 2: "laplace_fp64", 3: "laplace_c64", 4: "plain_df",
    5: "laplace_c64_unit", 6: "plain_fp64_unit", 7: "plain_c64_unit", 8: "plain_df_unit",
    9: "laplace_df_unit", 10: "laplace_df",
}

_lib = None
_lock = threading.Lock()


class EngineUnavailable(RuntimeError):
    """The CUDA engine is not built or no GPU is visible (there is no CPU path)."""


def load():
    """Loads the engine library (building nothing); raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise EngineUnavailable(
                    "piquasso_gb300 CUDA engine not built (%s missing); run "
                    "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
            lib = ctypes.CDLL(LIB_PATH)
            for name, (args, res) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.argtypes = args
                fn.restype = res
            _lib = lib
            _apply_tuning_cache()
    return _lib


def _apply_tuning_cache():
    """Fills the engine's autotuned-settings table from the tuning cache of
    this GPU and library version (piquasso_gb300.autotune), if there is one;
    without a visible GPU, or with PQG_TUNING=off, nothing is loaded."""
    if os.environ.get("PQG_TUNING", "").lower() in ("off", "0", "none"):
        return
    try:
        from . import autotune

        autotune.apply_cache(_lib)
    except Exception:  # noqa: BLE001  (a missing or unreadable cache leaves the defaults)
        pass


def last_error() -> str:
    return load().pqg_last_error().decode(errors="replace")


def kernel_launches() -> int:
    return int(load().pqg_kernel_launches())


def last_timing():
    """Event timing of this thread's last call: dict with walk_ms (walk kernel),
    device_ms (queue reset + walk + reductions), steps, flops and the bytes
    copied host-to-device / device-to-host."""
    v = [ctypes.c_double(0.0) for _ in range(6)]
    load().pqg_last_timing(*[ctypes.byref(x) for x in v])
    keys = ("walk_ms", "device_ms", "steps", "flops", "h2d_bytes", "d2h_bytes")
    return {k: x.value for k, x in zip(keys, v)}


def last_walk_kernel():
    """(table name, exact column count) of the walk kernel this thread's last
    call launched, or (None, 0) when it needed no walk."""
    t, n = ctypes.c_int32(0), ctypes.c_int32(0)
    load().pqg_last_walk_kernel(ctypes.byref(t), ctypes.byref(n))
    return (WALK_TABLES.get(t.value), n.value) if t.value >= 0 else (None, 0)


def check_tc_status():
    """Raises if a tensor-core kernel (the MLP GEMM or the fused proposal
    step) gave up a bounded wait since the last check (its results are then
    not to be trusted); clears the flag."""
    code = ctypes.c_int32(0)
    st = load().pqg_mlp_tc_status(ctypes.byref(code))
    if st:
        raise RuntimeError(last_error())
    if code.value:
        raise RuntimeError("a tensor-core kernel gave up a bounded wait (code %d)" % code.value)


def set_tuning(items_per_smsp=0, p_max=0, seed_steps=0):
    """Planner knobs (0 restores the default); see include/pqperm_gb300.h."""
    st = load().pqg_set_tuning(int(items_per_smsp), int(p_max), int(seed_steps))
    if st:
        raise ValueError(last_error())


def set_blocks_per_sm(blocks=0):
    """Process-wide cap on the walk's resident blocks per SM (0: as many as
    fit, or the autotuned value)."""
    st = load().pqg_set_blocks_per_sm(int(blocks))
    if st:
        raise ValueError(last_error())


def tuning_count():
    n = ctypes.c_int64(0)
    load().pqg_tuning_count(ctypes.byref(n))
    return n.value


def device_info():
    """(device name, SM count) of the engine's GPU; raises without one."""
    buf = ctypes.create_string_buffer(256)
    sms = ctypes.c_int32(0)
    st = load().pqg_device_info(buf, 256, ctypes.byref(sms))
    if st:
        raise EngineUnavailable(last_error())
    return buf.value.decode(errors="replace"), sms.value


def get_tuning():
    v = [ctypes.c_int64(0) for _ in range(3)]
    load().pqg_get_tuning(*[ctypes.byref(x) for x in v])
    return {"items_per_smsp": v[0].value, "p_max": v[1].value, "seed_steps": v[2].value}
