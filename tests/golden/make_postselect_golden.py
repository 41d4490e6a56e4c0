"""Generates tests/golden/sampler_postselect_seeded.json by running the
reference's own postselected samplers.

The reference package cannot be imported here (numba and blackbird are
missing), so this script loads the reference's
piquasso/_simulators/passive/sampling.py file unmodified. Its imports resolve to:

* the reference's own piquasso/_math/polynomial.py and piquasso/api/exceptions.py;
* to_first_quantized and to_second_quantized from piquasso/_math/indices.py,
  taken from that file's syntax tree with numba's ``njit`` as the identity;
* placeholders for the Fock-basis, marginal and loop-hafnian helpers, which
  are off the sampling paths run here.

The samplers are driven by the reference's compiled ``permanent_laplace``
(oracle/build_ref.sh), exactly as ``particle_number_measurement`` drives them
(passive/simulation_steps.py:239-369): ``generate_samples`` with
``reject_condition = lambda: config.rng.uniform() > s_0^2`` for uniform loss,
``generate_lossy_samples`` for non-uniform loss, and
``uniform_particle_overlap`` for partially distinguishable photons.
``config`` carries ``seed_sequence``, ``rng = default_rng(seed_sequence)``
(piquasso/api/config.py:159) and ``use_dask = False``.

Runs only where the reference source tree is present (PQ_REFERENCE_DIR, else
a directory named ``reference`` beside this repository).

Usage: python tests/golden/make_postselect_golden.py
"""

import ast
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


def _module(name, path=None, **attrs):
    m = types.ModuleType(name)
    if path is not None:
        m.__path__ = []
    m.__dict__.update(attrs)
    sys.modules[name] = m
    return m


def _exec_file(name, relpath):
    m = _module(name)
    m.__file__ = os.path.join(REF, relpath)
    exec(compile(open(m.__file__).read(), m.__file__, "exec"), m.__dict__)
    return m


def _functions_of(relpath, names, globs):
    src = open(os.path.join(REF, relpath)).read()
    fns = [n for n in ast.parse(src).body if isinstance(n, ast.FunctionDef) and n.name in names]
    exec(compile(ast.Module(body=fns, type_ignores=[]), relpath, "exec"), globs)
    return {n: globs[n] for n in names}


def load_ref_sampling():
    """The reference's sampling module, loaded with its off-path imports
    replaced.  sys.modules is restored afterwards, so the compiled reference
    package (oracle/_ref) stays importable."""
    saved = dict(sys.modules)
    try:
        for k in [k for k in sys.modules if k == "piquasso" or k.startswith("piquasso.")]:
            del sys.modules[k]
        _module("piquasso", path=True)
        _module("piquasso.api", path=True)
        _exec_file("piquasso.api.exceptions", "piquasso/api/exceptions.py")
        _module("piquasso._math", path=True)
        _exec_file("piquasso._math.polynomial", "piquasso/_math/polynomial.py")
        nb = types.SimpleNamespace(njit=lambda *a, **k: a[0] if a and callable(a[0]) else (lambda f: f),
                                   int64=np.int64)
        idx = _functions_of("piquasso/_math/indices.py", ["to_first_quantized", "to_second_quantized"],
                            {"np": np, "nb": nb})
        _module("piquasso._math.indices", **idx)
        _module("piquasso._math.fock", get_fock_space_basis=None, get_postselected_fock_basis=None)
        _module("piquasso._simulators", path=True)
        _module("piquasso._simulators.passive", path=True)
        _module("piquasso._simulators.passive.marginal", get_binomial_moments=None,
                get_single_marginal_probability_from_binomial_moments=None)
        _module("piquasso._simulators.passive.probabilities",
                get_lossy_partially_distinguishable_detection_probabilities=None)
        mod = types.ModuleType("piquasso._simulators.passive.sampling")
        mod.__package__ = "piquasso._simulators.passive"
        mod.__file__ = os.path.join(REF, "piquasso/_simulators/passive/sampling.py")
        sys.modules[mod.__name__] = mod
        exec(compile(open(mod.__file__).read(), mod.__file__, "exec"), mod.__dict__)
        exc = sys.modules["piquasso.api.exceptions"]
        return mod, exc
    finally:
        sys.modules.clear()
        sys.modules.update(saved)


def haar(d, seed):
    rng = np.random.default_rng(seed)
    z = (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(2.0)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def mat(a):
    a = np.asarray(a)
    return {"dtype": str(a.dtype), "shape": list(a.shape), "re": np.real(a).tolist(), "im": np.imag(a).tolist()}


# name, input, matrix, postselected modes, photons, overlap, shots, seed
def cases():
    U5, U5b, U6 = haar(5, 11), haar(5, 12), haar(6, 13)
    lossy = haar(5, 14) @ np.diag([0.95, 0.9, 0.8, 0.7, 0.6]) @ haar(5, 15)
    return [
        ("lossless_one_mode", [1, 1, 1, 0, 0], U5, (0,), (1,), None, 30, 123),
        ("lossless_two_modes_multiphoton", [2, 1, 1, 0, 1], U5b, (1, 3), (1, 0), None, 30, 7),
        ("lossless_zero_photons", [1, 1, 0, 1, 0, 1], U6, (5,), (0,), None, 30, 42),
        ("uniform_loss", [1, 1, 1, 1, 0], np.sqrt(0.8) * U5, (0,), (1,), None, 30, 5),
        ("nonuniform_loss", [1, 1, 1, 0, 0], lossy, (2,), (1,), None, 20, 9),
        ("overlap", [1, 1, 1, 0, 0], np.sqrt(0.95) * U5, (0,), (1,), 0.5, 30, 3),
        ("overlap_multiphoton_two_modes", [2, 1, 0, 1, 0], np.sqrt(0.97) * U5b, (0, 1), (1, 0), 0.7, 30, 17),
        ("overlap_uniform_loss", [1, 1, 1, 1, 0], np.sqrt(0.9) * U5, (0, 2), (1, 0), 0.6, 25, 21),
    ]


def run(samp, perm_laplace, inp, M, modes, photons, overlap, shots, seed, max_trials=1000):
    """particle_number_measurement's sampling branch for these arguments."""
    inp = np.asarray(inp, dtype=int)
    config = types.SimpleNamespace(seed_sequence=seed, rng=np.random.default_rng(seed), use_dask=False)
    ps = (tuple(modes), tuple(photons), max_trials)
    sv = np.linalg.svd(M, compute_uv=False)
    if not np.all(np.isclose(sv, sv[0])):
        return samp.generate_lossy_samples(inp, shots, perm_laplace, M, postselect_data=ps, config=config)
    T = sv[0] ** 2
    reject = (lambda: False) if np.isclose(sv[0], 1.0) else (lambda: config.rng.uniform() > T)
    return samp.generate_samples(inp, shots, perm_laplace, M, reject_condition=reject, postselect_data=ps,
                                 uniform_particle_overlap=overlap, config=config)


def main():
    oracle.build.build()
    ref = oracle.reference_module()
    if ref is None:
        raise SystemExit("reference module not built (oracle/build_ref.sh needs the reference sources)")
    samp, exc = load_ref_sampling()
    out = {"source": "piquasso/_simulators/passive/sampling.py: generate_samples, generate_lossy_samples with "
                     "postselect_data (_generate_sample_with_postselect, "
                     "_generate_sample_with_postselect_and_uniform_overlap)",
           "cases": []}
    for name, inp, M, modes, photons, overlap, shots, seed in cases():
        S = run(samp, ref.permanent_laplace, inp, M, modes, photons, overlap, shots, seed)
        out["cases"].append({"name": name, "input": list(inp), "matrix": mat(M), "modes": list(modes),
                             "photons": list(photons), "overlap": overlap, "shots": shots, "seed": seed,
                             "samples": [[int(x) for x in s] for s in S]})
        print(name, len(S), S[:3])
    # Lossless partially distinguishable photons with postselection: the
    # distinguishable photons' loss weight 1 - sum_i |U[i, j]|^2
    # (sampling.py:617-619) rounds to about -1e-16 for a unitary, and numpy's
    # choice rejects the negative weight.  Recorded, not reproduced.
    try:
        run(samp, ref.permanent_laplace, [1, 1, 1, 0, 0], haar(5, 11), (0,), (1,), 0.5, 30, 3)
        out["lossless_overlap"] = {"raises": None}
    except ValueError as e:
        out["lossless_overlap"] = {"raises": "ValueError: %s" % e}
    # the trial limit: five photons asked for in one mode of a four-photon state
    try:
        run(samp, ref.permanent_laplace, [2, 0, 2, 0], haar(4, 16), (0,), (5,), None, 1, 0, max_trials=10)
        raise SystemExit("the trial limit did not trigger")
    except exc.InvalidSimulation as e:
        out["trial_limit"] = {"input": [2, 0, 2, 0], "matrix": mat(haar(4, 16)), "modes": [0], "photons": [5],
                              "max_trials": 10, "exception": "InvalidSimulation", "message": str(e)}
    with open(os.path.join(HERE, "sampler_postselect_seeded.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote sampler_postselect_seeded.json")


if __name__ == "__main__":
    main()
