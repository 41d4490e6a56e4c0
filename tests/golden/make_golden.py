"""Generates the golden fixtures in tests/golden/ from the reference itself.

Runs only where the reference source tree is present (PQ_REFERENCE_DIR, else
a directory named ``reference`` beside this repository) and its permanent module has
been compiled by oracle/build_ref.sh.  Outputs (JSON, complex numbers as
[re, im] pairs):

* ``permanent_known_answers.json`` — every call that the reference's own
  tests/_math/test_permanent.py makes to ``permanent`` while those tests run
  (their own assertions included), with the reference module's result.
* ``jax_unit_cases.json`` — the same for the numpy-only cases of
  tests/jax_extensions/test_permanent_unit.py, run with ``perm`` bound to the
  reference's CPU permanent (jax is not installed).
* ``sampler_seeded.json`` — unitary, input, seed and expected samples of
  tests/_simulators/passive/test_measurements.py::test_boson_sampling_seeded
  (read from the file's syntax tree), checked against oracle.sampler driven
  by the reference module's permanent_laplace; ``generated_samples`` holds the
  samples in generation order, before Result.samples bins and shuffles them.
* ``sampler_lossy_seeded.json`` — the two seeded lossy-sampling goldens of the same
  test file (non-uniform singular values through the SVD dilation; uniform
  ones through the per-photon reject condition), reproduced by oracle.sampler
  over the reference module's permanent_laplace.
* ``lxeb_values.json`` — the reference's Haar-averaged LXEB reference values
  (piquasso/lxeb.py, loaded from its file) on a grid of photon and mode
  numbers, and the value its tests/test_lxeb.py asserts.
* ``random_cases.json`` — seeded random permanent and Laplace cases
  (complex128 and complex64) with the reference module's outputs.
* ``config_14.json`` — the 14x14 parity cases: leading 14x14 block of a seeded
  28x28 Haar unitary, all-ones multiplicities and a repeated-row case.
* ``grad_cases.json`` — every gradient the reference's own
  tests/jax_extensions/test_permanent_grad.py asks for through
  ``jax.grad(perm, holomorphic=True)``, answered by oracle.grad_perm over the
  reference module's permanent and checked by those tests' own golden
  assertions (the parts that need jax.jacobian are not run: jax is not
  installed), plus seeded random cases (repeated rows and columns, non-square).

Usage: python tests/golden/make_golden.py
"""

import ast
import inspect
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("PQ_REFERENCE_DIR") or os.path.join(os.path.dirname(REPO), "reference")
sys.path.insert(0, REPO)

import oracle  # noqa: E402
from oracle import sampler as osampler  # noqa: E402


def cpx(z):
    z = complex(z)
    return [z.real, z.imag]


def mat(a):
    a = np.asarray(a)
    return {"dtype": str(a.dtype), "shape": list(a.shape), "re": np.real(a).tolist(), "im": np.imag(a).tolist()}


class Recorder:
    def __init__(self, fn):
        self.fn = fn
        self.calls = []

    def __call__(self, matrix, rows=None, cols=None):
        out = self.fn(matrix, rows=rows, cols=cols)
        self.calls.append({
            "matrix": mat(np.asarray(matrix)),
            "rows": np.asarray(rows).astype(int).tolist(),
            "cols": np.asarray(cols).astype(int).tolist(),
            "result": cpx(out),
            "result_dtype": str(np.asarray(out).dtype),
        })
        return out


def load_ref_linalg():
    src = open(os.path.join(REF, "piquasso/_math/linalg.py")).read()
    tree = ast.parse(src)
    fn = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "assym_reduce"][0]
    mod = types.ModuleType("ref_linalg")
    mod.np = np
    exec(compile(ast.Module(body=[fn], type_ignores=[]), "linalg.py", "exec"), mod.__dict__)
    return mod


def run_test_module(path, perm_name, perm_fn, extra_globals):
    """Executes the module's test functions that take no fixtures."""
    src = open(path).read()
    tree = ast.parse(src)
    body = [n for n in tree.body if not isinstance(n, (ast.Import, ast.ImportFrom))
            and not (isinstance(n, ast.Expr) and isinstance(getattr(n, "value", None), ast.Call))
            and not isinstance(n, ast.Assign)]
    g = {"np": np, perm_name: perm_fn, "__name__": "golden_run"}
    g.update(extra_globals)
    exec(compile(ast.Module(body=body, type_ignores=[]), path, "exec"), g)
    ran, skipped = [], []
    for name, obj in list(g.items()):
        if not name.startswith("test_") or not callable(obj):
            continue
        if inspect.signature(obj).parameters:
            skipped.append(name)
            continue
        try:
            obj()
            ran.append(name)
        except Exception as e:  # cases that need jax or raise on purpose
            skipped.append("%s (%s)" % (name, type(e).__name__))
    return ran, skipped


class _PytestStub:
    @staticmethod
    def raises(exc):
        class Ctx:
            def __enter__(self):
                return self

            def __exit__(self, t, v, tb):
                if t is None:
                    raise AssertionError("expected an exception")
                return issubclass(t, exc)
        return Ctx()

    class mark:
        @staticmethod
        def monkey(f):
            return f

        @staticmethod
        def parametrize(*a, **k):
            return lambda f: f


def gen_known_answers(ref):
    rec = Recorder(ref.permanent)
    lin = load_ref_linalg()
    ran, skipped = run_test_module(os.path.join(REF, "tests/_math/test_permanent.py"), "permanent", rec,
                                   {"assym_reduce": lin.assym_reduce, "pytest": _PytestStub})
    return {"source": "tests/_math/test_permanent.py", "tests_run": ran, "tests_skipped": skipped,
            "calls": rec.calls}


def gen_jax_cases(ref):
    calls = []

    def perm(A, rows, cols):
        A = np.asarray(A)
        if not np.iscomplexobj(A):
            raise TypeError("real matrix")  # the FFI path rejects real input
        out = ref.permanent(A, rows=np.asarray(rows).astype(np.int64), cols=np.asarray(cols).astype(np.int64))
        calls.append({"matrix": mat(A), "rows": np.asarray(rows).astype(int).tolist(),
                      "cols": np.asarray(cols).astype(int).tolist(), "result": cpx(out),
                      "result_dtype": str(np.asarray(out).dtype)})
        return out

    jnp_stub = types.SimpleNamespace(array=np.array, asarray=np.asarray, uint64=np.uint64, uint32=np.uint32,
                                     complex128=np.complex128, ones=np.ones, zeros=np.zeros, eye=np.eye)
    ran, skipped = run_test_module(os.path.join(REF, "tests/jax_extensions/test_permanent_unit.py"), "perm", perm,
                                   {"pytest": _PytestStub, "jnp": jnp_stub, "jax": types.SimpleNamespace()})
    return {"source": "tests/jax_extensions/test_permanent_unit.py", "tests_run": ran, "tests_skipped": skipped,
            "calls": calls}


def gen_sampler(ref):
    path = os.path.join(REF, "tests/_simulators/passive/test_measurements.py")
    tree = ast.parse(open(path).read())
    fn = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == "test_boson_sampling_seeded"][0]
    vals = {}
    for node in ast.walk(fn):
        if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name):
            name = node.targets[0].id
            if name in ("seed_sequence", "expected_samples"):
                vals[name] = ast.literal_eval(node.value)
            if name == "U":
                vals["U"] = np.array(ast.literal_eval(node.value.args[0]))
        if isinstance(node, ast.Call) and getattr(node.func, "attr", None) == "NumberState":
            vals["input"] = ast.literal_eval(node.args[0])
        if isinstance(node, ast.keyword) and node.arg == "shots":
            vals["shots"] = ast.literal_eval(node.value)
    samples = osampler.generate_samples(np.array(vals["input"]), vals["shots"], ref.permanent_laplace,
                                        vals["U"], vals["seed_sequence"])
    expected = [tuple(s) for s in vals["expected_samples"]]
    got = osampler.result_samples(samples, vals["seed_sequence"])
    assert got == expected, "restated sampler does not reproduce the reference golden"
    return {"source": "tests/_simulators/passive/test_measurements.py::test_boson_sampling_seeded",
            "U": mat(vals["U"]), "input": vals["input"], "seed": vals["seed_sequence"], "shots": vals["shots"],
            "generated_samples": [list(s) for s in samples],
            "expected_samples": vals["expected_samples"]}


def gen_lossy_sampler(ref):
    """The two seeded lossy goldens of tests/_simulators/passive/test_measurements.py:
    non-uniform singular values (SVD dilation) and uniform ones (reject
    condition on the configuration generator)."""
    path = os.path.join(REF, "tests/_simulators/passive/test_measurements.py")
    tree = ast.parse(open(path).read())
    cases = []
    for name in ("test_LossyInterferometer_boson_sampling_seeded",
                 "test_LossyInterferometer_boson_sampling_uniform_losses"):
        fn = [n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == name][0]
        vals = {}
        for node in ast.walk(fn):
            if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name):
                t = node.targets[0].id
                if t in ("seed_sequence", "expected_samples"):
                    vals[t] = ast.literal_eval(node.value)
                if t in ("U", "singular_values"):  # np.array(<literal list expression>)
                    vals[t] = np.array(eval(ast.unparse(node.value.args[0]), {"__builtins__": {}}))
                if t == "lossy_interferometer_matrix":
                    vals["formula"] = ast.unparse(node.value)
            if isinstance(node, ast.Call) and getattr(node.func, "attr", None) == "NumberState":
                vals["input"] = ast.literal_eval(node.args[0])
            if isinstance(node, ast.keyword) and node.arg == "shots":
                vals["shots"] = ast.literal_eval(node.value)
        M = eval(vals["formula"], {"np": np, "U": vals["U"], "singular_values": vals["singular_values"]})
        sv = np.linalg.svd(M, compute_uv=False)
        inp = np.array(vals["input"])
        if np.all(np.isclose(sv, sv[0])):
            kind = "uniform"
            samples = osampler.generate_samples(inp, vals["shots"], ref.permanent_laplace, M, vals["seed_sequence"],
                                                transmission=float(sv[0] ** 2))
        else:
            kind = "nonuniform"
            samples = osampler.generate_lossy_samples(inp, vals["shots"], ref.permanent_laplace, M,
                                                      vals["seed_sequence"])
        expected = [tuple(x) for x in vals["expected_samples"]]
        got = osampler.result_samples(samples, vals["seed_sequence"])
        assert got == expected, "restated %s lossy sampler does not reproduce %s" % (kind, name)
        cases.append({"source": "tests/_simulators/passive/test_measurements.py::" + name, "kind": kind,
                      "matrix": mat(M), "input": vals["input"], "seed": vals["seed_sequence"],
                      "shots": vals["shots"], "transmission": float(sv[0] ** 2) if kind == "uniform" else None,
                      "generated_samples": [list(map(int, x)) for x in samples],
                      "expected_samples": vals["expected_samples"]})
    return {"cases": cases}


def gen_lxeb():
    """Outputs of the reference's own piquasso/lxeb.py (a dependency-free
    module, loaded from its file) on a grid of (n, m), plus the values its
    tests/test_lxeb.py asserts."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("ref_lxeb", os.path.join(REF, "piquasso/lxeb.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    grid = []
    for n in range(0, 31):
        for m in (1, 2, 3, 5, 8, 16, 40, 48, 100):
            grid.append({"n": n, "m": m, "value": mod.lxe_ref_boson_sampling(n, m)})
    return {"source": "piquasso/lxeb.py", "boson_sampling": grid,
            "test_values": [{"n": 10, "m": 3, "value": 0.018798373343827918}]}


def haar(d, seed):
    rng = np.random.default_rng(seed)
    Z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2)
    Q, R = np.linalg.qr(Z)
    return Q * (np.diag(R) / np.abs(np.diag(R)))


def gen_random(ref):
    rng = np.random.default_rng(2024)
    perm_cases, lap_cases = [], []
    for t in range(60):
        nr = int(rng.integers(1, 7))
        nc = int(rng.integers(1, 7))
        n = int(rng.integers(0, 9))
        rows = np.bincount(rng.integers(0, nr, n), minlength=nr)
        cols = np.bincount(rng.integers(0, nc, n), minlength=nc)
        A = rng.normal(size=(nr, nc)) + 1j * rng.normal(size=(nr, nc))
        dt = np.complex64 if t % 3 == 0 else np.complex128
        A = A.astype(dt)
        out = ref.permanent(A, rows=rows, cols=cols)
        perm_cases.append({"matrix": mat(A), "rows": rows.tolist(), "cols": cols.tolist(), "result": cpx(out),
                           "result_dtype": str(out.dtype), "dd": cpx(oracle.permanent(A.astype(np.complex128), rows, cols)),
                           "perm_abs": oracle.perm_abs(A.astype(np.complex128), rows, cols)})
    for t in range(40):
        nr = int(rng.integers(1, 7))
        nc = int(rng.integers(1, 7))
        cols = rng.integers(1, 3, nc)
        n = int(cols.sum()) - 1
        rows = np.bincount(rng.integers(0, nr, n), minlength=nr)
        A = rng.normal(size=(nr, nc)) + 1j * rng.normal(size=(nr, nc))
        dt = np.complex64 if t % 3 == 0 else np.complex128
        A = A.astype(dt)
        out = ref.permanent_laplace(A, rows, cols)
        lap_cases.append({"matrix": mat(A), "rows": rows.tolist(), "cols": cols.tolist(),
                          "result": [cpx(z) for z in out], "result_dtype": str(out.dtype),
                          "dd": [cpx(z) for z in oracle.permanent_laplace_dd(A.astype(np.complex128), rows, cols)]})
    return {"permanent": perm_cases, "laplace": lap_cases}


def gen_config14(ref):
    U = haar(28, 0)[:14, :14].copy()
    ones = np.ones(14, dtype=int)
    rep_rows = np.array([2, 2, 1, 1, 1, 1] + [0] * 8)
    rep_cols = np.array([1] * 8 + [0] * 6)
    cases = []
    for rows, cols, label in ((ones, ones, "all-ones"), (rep_rows, rep_cols, "repeated-rows")):
        for dt in (np.complex128, np.complex64):
            A = U.astype(dt)
            out = ref.permanent(A, rows=rows, cols=cols)
            A128 = A.astype(np.complex128)
            hi, lo = oracle.permanent_dd(A128, rows, cols)
            cases.append({"label": label, "matrix": mat(A), "rows": rows.tolist(), "cols": cols.tolist(),
                          "result": cpx(out), "result_dtype": str(out.dtype), "dd_hi": cpx(hi), "dd_lo": cpx(lo),
                          "perm_abs": oracle.perm_abs(A128, rows, cols)})
    return {"haar_seed": 0, "haar_dim": 28, "cases": cases}


class _JacobianSkipped(Exception):
    pass


def gen_grad_cases(ref):
    calls = []

    def grad(fn, holomorphic=False):
        assert holomorphic

        def g(A, rows, cols):
            A = np.asarray(A, dtype=np.complex128)
            rows = np.asarray(rows).astype(np.int64)
            cols = np.asarray(cols).astype(np.int64)
            G = oracle.grad_perm(A, rows, cols, perm=lambda M, r, c: ref.permanent(M, rows=r, cols=c))
            calls.append({"test": sys._getframe(1).f_code.co_name, "matrix": mat(A), "rows": rows.tolist(),
                          "cols": cols.tolist(), "grad": mat(G)})
            return G
        return g

    def jacobian(*a, **k):
        raise _JacobianSkipped()

    jax_stub = types.SimpleNamespace(grad=grad, jacobian=jacobian,
                                     numpy=types.SimpleNamespace(array=np.array, uint64=np.uint64,
                                                                 complex128=np.complex128))
    ran, skipped = run_test_module(os.path.join(REF, "tests/jax_extensions/test_permanent_grad.py"), "perm",
                                   None, {"pytest": _PytestStub, "jax": jax_stub})
    # a test that reached jax.jacobian passed every golden assertion before it
    # (only tests that asked for a gradient count: the others check nothing here)
    asked = {c["test"] for c in calls}
    golden = [t for t in ran + [t.split(" ")[0] for t in skipped if "_JacobianSkipped" in t] if t in asked]
    skipped = [t for t in skipped if "_JacobianSkipped" not in t] + sorted(
        set(ran + [t.split(" ")[0] for t in skipped]) - asked)
    rng = np.random.default_rng(77)
    rand = []
    for t in range(24):
        nr = int(rng.integers(1, 6))
        nc = int(rng.integers(1, 6))
        n = int(rng.integers(1, 8))
        rows = np.bincount(rng.integers(0, nr, n), minlength=nr)
        cols = np.bincount(rng.integers(0, nc, n), minlength=nc)
        A = rng.normal(size=(nr, nc)) + 1j * rng.normal(size=(nr, nc))
        G = oracle.grad_perm(A, rows, cols, perm=lambda M, r, c: ref.permanent(M, rows=r, cols=c))
        rand.append({"matrix": mat(A), "rows": rows.tolist(), "cols": cols.tolist(), "grad": mat(G)})
    return {"source": "tests/jax_extensions/test_permanent_grad.py", "tests_golden_checked": golden,
            "tests_skipped": skipped, "calls": calls, "random": rand}


def main():
    oracle.build.build()
    ref = oracle.reference_module()
    if ref is None:
        raise SystemExit("reference module not built (oracle/build_ref.sh needs the reference sources)")
    outputs = {
        "permanent_known_answers.json": gen_known_answers(ref),
        "jax_unit_cases.json": gen_jax_cases(ref),
        "sampler_seeded.json": gen_sampler(ref),
        "random_cases.json": gen_random(ref),
        "config_14.json": gen_config14(ref),
        "grad_cases.json": gen_grad_cases(ref),
        "sampler_lossy_seeded.json": gen_lossy_sampler(ref),
        "lxeb_values.json": gen_lxeb(),
    }
    for name, obj in outputs.items():
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(obj, f, indent=1)
        extra = ""
        if "tests_run" in obj:
            extra = " ran=%d skipped=%s" % (len(obj["tests_run"]), obj["tests_skipped"])
        if "tests_golden_checked" in obj:
            extra = " golden=%s skipped=%s" % (obj["tests_golden_checked"], obj["tests_skipped"])
        print("wrote", name, extra)


if __name__ == "__main__":
    main()
