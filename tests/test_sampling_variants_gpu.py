"""GPU: the lossy and partially distinguishable samplers and the batched
detection probabilities.

* the reference-RNG sampler reproduces the reference's two seeded lossy
  goldens (non-uniform loss through the SVD dilation, uniform loss through the
  per-photon reject condition), directly and through ``sample``'s dispatch;
* with loss and uniform particle overlap together it draws exactly the
  samples of the CPU restatement (oracle.sampler, same random-number order);
* Hong-Ou-Mandel: two photons of overlap x on a 50:50 beamsplitter give
  P(1,1) = (1 - x^2)/2 under the reference's separation model;
* the batched sampler's mean output occupations equal sum_i |M_ji|^2 n_i;
* detection probabilities match the oracle's permanents, sum to the norm of
  the input state's fixed-photon-number part, and the mean ideal probability
  of exact samples matches sum_y p(y)^2.

Statistical tolerances are 5 standard errors (seeded, so deterministic).
"""

import itertools
import math

import numpy as np
import pytest

import oracle
from conftest import as_matrix, haar_unitary, load_golden
from oracle import sampler as osampler

pytestmark = pytest.mark.gpu


def test_lossy_goldens(engine):
    from piquasso_gb300 import sampling

    g = load_golden("sampler_lossy_seeded.json")
    for c in g["cases"]:
        M = as_matrix(c["matrix"]).astype(np.complex128)
        inp = np.array(c["input"])
        if c["kind"] == "uniform":
            got = sampling.generate_samples(inp, c["shots"], M, c["seed"], transmission=c["transmission"])
        else:
            got = sampling.generate_lossy_samples(inp, c["shots"], M, c["seed"])
        assert [list(s) for s in got] == c["generated_samples"], c["kind"]
        assert [list(s) for s in sampling.result_samples(got, c["seed"])] == c["expected_samples"]
        via = sampling.sample(inp, c["shots"], M, c["seed"])
        assert [list(s) for s in via] == c["generated_samples"]


def test_overlap_and_loss_match_restatement(engine):
    from piquasso_gb300 import sampling

    U = haar_unitary(4, 8) * np.sqrt(0.8)
    inp = np.array([2, 1, 1, 0])
    got = sampling.generate_samples(inp, 40, U, 5, transmission=0.8, particle_overlap=0.6)
    want = osampler.generate_samples(inp, 40, oracle.permanent_laplace_dd, U, 5, transmission=0.8, overlap=0.6)
    assert got == want


@pytest.mark.parametrize("x", [0.0, 0.5, 1.0])
def test_hong_ou_mandel(engine, x):
    from piquasso_gb300 import sampling

    B = np.array([[1, 1], [1, -1]], dtype=np.complex128) / np.sqrt(2)
    p11 = (1 - x * x) / 2
    S = sampling.generate_samples_batched([1, 1], 20000, B, 3, particle_overlap=x)
    f = np.mean((S[:, 0] == 1) & (S[:, 1] == 1))
    assert abs(f - p11) <= 5 * np.sqrt(max(p11 * (1 - p11), 1e-4) / 20000) + 1e-12
    R = sampling.generate_samples([1, 1], 600, B, 4, particle_overlap=x)
    fr = np.mean([s == (1, 1) for s in R])
    assert abs(fr - p11) <= 5 * np.sqrt(max(p11 * (1 - p11), 1e-3) / 600) + 1e-12
    if x == 1.0:
        assert f == 0.0 and fr == 0.0


@pytest.mark.parametrize("case", ["uniform", "nonuniform", "overlap"])
def test_batched_mean_occupations(engine, case):
    from piquasso_gb300 import sampling

    d = 6
    U = haar_unitary(d, 21)
    inp = np.array([1, 1, 1, 1, 0, 0])
    if case == "uniform":
        M = U * 0.9
    elif case == "nonuniform":
        M = U @ np.diag([0.95, 0.9, 0.8, 0.7, 0.6, 0.5]) @ haar_unitary(d, 22)
    else:
        M = U
    S = np.asarray(sampling.sample(inp, 12000, M, 9, particle_overlap=0.5 if case == "overlap" else None,
                                   batched=True))
    mean = (np.abs(M) ** 2) @ inp
    se = S.std(axis=0) / np.sqrt(len(S))
    assert np.all(np.abs(S.mean(axis=0) - mean) <= 5 * se + 1e-3), (S.mean(axis=0), mean)
    if case == "uniform":
        tot = S.sum(axis=1)
        assert abs(tot.mean() - 4 * 0.81) <= 5 * tot.std() / np.sqrt(len(S))


def test_detection_probabilities(engine):
    from piquasso_gb300 import probabilities, sampling

    d, n = 5, 3
    U = haar_unitary(d, 6)
    inp = np.array([1, 1, 1, 0, 0])
    pats = np.array([c for c in itertools.product(range(n + 1), repeat=d) if sum(c) == n])
    p = probabilities.detection_probabilities(U, pats, inp)
    assert abs(p.sum() - 1.0) < 1e-12
    for y in pats[::7]:
        amp = oracle.permanent(U, y, inp) / np.sqrt(np.prod([float(math.factorial(k)) for k in y]))
        assert abs(abs(amp) ** 2 - probabilities.get_particle_detection_probability(U, y, inp)) < 1e-13
    # a superposition of two inputs with 3 photons and one with 2 photons
    X = np.array([[1, 1, 1, 0, 0], [0, 2, 0, 1, 0], [1, 1, 0, 0, 0]])
    c = np.array([0.6, 0.48j, 0.64])
    p2 = probabilities.detection_probabilities(U, pats, X, c)
    assert abs(p2.sum() - (0.36 + 0.2304)) < 1e-12
    # LXEB: the mean ideal probability of exact samples estimates sum_y p(y)^2
    S = sampling.generate_samples_batched(inp, 20000, U, 2)
    sc = probabilities.lxeb_score(U, inp, S)
    ps = probabilities.detection_probabilities(U, S, inp)
    assert abs(sc["mean_probability"] - (p ** 2).sum()) <= 5 * ps.std() / np.sqrt(len(S))
    assert sc["reference"] == probabilities.lxe_ref_boson_sampling(3, 5)
