"""CPU tests: the oracle pinned against the reference's golden vectors.

The double-double restatement (oracle/perm_oracle.cpp) and the port of the
reference's CPU method (oracle/perm_port.cpp) must reproduce every fixture in
tests/golden/, which were recorded from the reference itself.
"""

import numpy as np
import pytest

import oracle
from conftest import as_complex, as_matrix, haar_unitary, load_golden
from oracle import sampler as osampler


@pytest.fixture(scope="module", autouse=True)
def _built():
    oracle.build.build(with_reference=False)


@pytest.mark.parametrize("fixture", ["permanent_known_answers.json", "jax_unit_cases.json"])
def test_oracle_reproduces_reference_known_answers(fixture):
    data = load_golden(fixture)
    assert len(data["calls"]) >= 10
    for case in data["calls"]:
        A = as_matrix(case["matrix"]).astype(np.complex128)
        ref = as_complex(case["result"])
        dd = oracle.permanent(A, case["rows"], case["cols"])
        tol = max(1e-10 * abs(ref), 1e-14 * oracle.perm_abs(A, case["rows"], case["cols"]))
        if case["result_dtype"] == "complex64":
            tol = max(tol, 1e-6 * max(1.0, abs(ref)))
        assert abs(dd - ref) <= tol, (case["rows"], case["cols"], dd, ref)


def test_oracle_and_port_reproduce_random_reference_cases():
    data = load_golden("random_cases.json")
    for case in data["permanent"]:
        A = as_matrix(case["matrix"])
        ref = as_complex(case["result"])
        dd = oracle.permanent(A.astype(np.complex128), case["rows"], case["cols"])
        assert abs(dd - as_complex(case["dd"])) <= 1e-15 * max(1.0, abs(dd))
        port = complex(oracle.port_permanent(A, case["rows"], case["cols"]))
        if A.dtype == np.complex64:
            t = max(1e-4 * abs(dd), 2.0 ** -20 * case["perm_abs"])
            assert abs(port - ref) <= t
        else:
            t = max(1e-10 * abs(dd), 1e-14 * case["perm_abs"])
            assert abs(ref - dd) <= t
            assert abs(port - dd) <= t
    for case in data["laplace"]:
        A = as_matrix(case["matrix"])
        ref = np.array([as_complex(z) for z in case["result"]])
        dd = oracle.permanent_laplace_dd(A.astype(np.complex128), case["rows"], case["cols"])
        assert np.allclose(dd, np.array([as_complex(z) for z in case["dd"]]), rtol=1e-15, atol=1e-300)
        rt = 1e-4 if A.dtype == np.complex64 else 1e-10
        assert np.allclose(ref, dd, rtol=rt, atol=rt * 1e-2)
        port = oracle.port_laplace(A, case["rows"], case["cols"])
        assert np.allclose(port, dd, rtol=rt, atol=rt * 1e-2)


def test_oracle_config14():
    data = load_golden("config_14.json")
    for case in data["cases"]:
        A = as_matrix(case["matrix"]).astype(np.complex128)
        hi, lo = oracle.permanent_dd(A, case["rows"], case["cols"])
        want = as_complex(case["dd_hi"]) + as_complex(case["dd_lo"])
        assert abs((hi + lo) - want) <= 1e-15 * abs(want)
        if case["result_dtype"] == "complex128":
            t = max(1e-10 * abs(want), 1e-14 * case["perm_abs"])
            assert abs(as_complex(case["result"]) - want) <= t


def test_restated_sampler_reproduces_reference_golden():
    g = load_golden("sampler_seeded.json")
    U = as_matrix(g["U"])
    samples = osampler.generate_samples(np.array(g["input"]), g["shots"], oracle.permanent_laplace_dd, U, g["seed"])
    assert [list(s) for s in samples] == g["generated_samples"]
    assert [list(s) for s in osampler.result_samples(samples, g["seed"])] == g["expected_samples"]


def test_restated_lossy_samplers_reproduce_reference_goldens():
    """Non-uniform loss (SVD dilation) and uniform loss (per-photon reject
    condition) of tests/_simulators/passive/test_measurements.py."""
    g = load_golden("sampler_lossy_seeded.json")
    assert {c["kind"] for c in g["cases"]} == {"uniform", "nonuniform"}
    for c in g["cases"]:
        M = as_matrix(c["matrix"])
        inp = np.array(c["input"])
        if c["kind"] == "uniform":
            samples = osampler.generate_samples(inp, c["shots"], oracle.permanent_laplace_dd, M, c["seed"],
                                                transmission=c["transmission"])
        else:
            samples = osampler.generate_lossy_samples(inp, c["shots"], oracle.permanent_laplace_dd, M, c["seed"])
        assert [list(s) for s in samples] == c["generated_samples"], c["kind"]
        assert [list(s) for s in osampler.result_samples(samples, c["seed"])] == c["expected_samples"]


def test_oracle_identities():
    U = haar_unitary(10, 4)[:8, :8].copy()
    ones = np.ones(8, dtype=int)
    p = oracle.permanent(U, ones, ones)
    assert abs(oracle.permanent(U.T.copy(), ones, ones) - p) < 1e-14
    # repeated rows == explicit repetition (assym_reduce)
    rows = np.array([2, 0, 1, 3, 0, 1, 1, 0])
    cols = np.array([1, 1, 2, 0, 1, 1, 1, 1])
    ri = np.repeat(np.arange(8), rows)
    ci = np.repeat(np.arange(8), cols)
    B = U[np.ix_(ri, ci)]
    o = np.ones(len(ri), dtype=int)
    assert abs(oracle.permanent(U, rows, cols) - oracle.permanent(B, o, o)) < 1e-13
    with pytest.raises(ValueError):
        oracle.permanent(U, rows, ones + np.eye(8, dtype=int)[0])
