"""Exact boson sampling on the GPU (Clifford & Clifford algorithm B).

A drop-in for the reference's ``PassiveSimulator`` sampler
(piquasso/_simulators/passive/sampling.py:149-236, 711-753): lossless,
uniformly lossy (a per-photon reject condition), non-uniformly lossy (the
lossless sampler on an SVD dilation, sampling.py:110-146) and with uniform
partial distinguishability (sampling.py:328-418); ``sample`` dispatches as
the reference's passive/simulation_steps.py:315-369 does.  Every shot keeps its own ``np.random.default_rng(seed + idx)`` and
draws exactly the random numbers the reference draws, in the same order, so a
given seed reproduces the reference's samples.  What changes is the schedule:
all shots advance one photon at a time together, and each photon step is ONE
batched Laplace-permanent launch over every shot (``permanent_laplace_batch``)
instead of one CPU call per shot and step.

``result_samples`` reproduces ``Result.samples`` (piquasso/api/result.py:104-136):
the generated samples binned by first occurrence (piquasso/_utils.py:23-31),
expanded, then shuffled with ``random.Random(seed)``.
"""

import random

import numpy as np

from .permanent import permanent_laplace_batch, sampler_step_batch


def to_first_quantized(occupation_numbers):
    occ = np.asarray(occupation_numbers)
    return np.repeat(np.arange(len(occ)), occ).astype(occ.dtype)


def _pmf_batch(U, current_input, samples, laplace):
    """pmf[s, idx] of sampling.py:723-749 for every shot, with the reference's
    summation order: the terms over the nonzero input modes in increasing
    order, then the normalisation over idx in increasing order (``cumsum``
    adds left to right, as the reference's loop does).  Vectorised over shots
    with the same elementwise operations; a shot with fewer terms keeps its
    amplitude unchanged at the steps it does not take."""
    shots, d = samples.shape
    current_input = np.asarray(current_input)
    nzmask = current_input > 0
    terms = nzmask.sum(axis=1)
    # the nonzero input modes of every shot first, in increasing order
    order = np.argsort(~nzmask, axis=1, kind="stable")
    # empty output: the reference's Laplace vector is [1] (one entry), so one term
    empty = samples.sum(axis=1) == 0
    terms = np.where(empty, 1, terms)
    lap = np.asarray(laplace, dtype=np.complex128)
    Ut = np.ascontiguousarray(np.asarray(U).T)
    at = np.arange(shots)
    amp = np.zeros((shots, d), dtype=np.complex128)
    for t in range(int(terms.max(initial=0))):
        j = order[:, t]
        part = np.where(empty, 1.0 + 0.0j, lap[at, j])
        coef = current_input[at, j] * part
        stepped = amp + coef[:, None] * Ut[j]
        amp = np.where((t < terms)[:, None], stepped, amp)
    p = np.abs(amp) ** 2
    norm = np.cumsum(p, axis=1)[:, -1]
    return p / norm[:, None]


def _draw_from_pmf(pmf, u):
    """``rng.choice(np.arange(d), p=pmf[s])`` of every shot s, from one
    ``rng.random()`` per shot (u[s]), which is all the draw takes from the
    generator: numpy's Generator.choice with p and no size normalises the
    cumulative sum by its last entry and returns searchsorted(cdf, u,
    'right'), the number of entries <= u (sampling.py:752-753 of the
    reference makes that call)."""
    if np.isnan(pmf).any() or (pmf < 0).any():  # rng.choice refuses these; so does this draw
        raise ValueError("probabilities contain NaN or negative values")
    cdf = np.cumsum(pmf, axis=1)
    cdf /= cdf[:, -1:]
    return (cdf <= u[:, None]).sum(axis=1)


def _separate_particles(input_occupation, overlap, rng):
    """sampling.py:371-400 of the reference: per occupied input mode j, the
    number K of indistinguishable photons, drawn with weights
    C(n_j, k) x^k (1 - x)^(n_j - k) k!  (same floating-point formula)."""
    from scipy.special import comb, factorial

    d = len(input_occupation)
    indist = np.zeros(d, dtype=int)
    dist = np.zeros(d, dtype=int)
    for j, n_j in enumerate(input_occupation):
        if n_j == 0:
            continue
        weights = np.array([comb(n_j, k) * (overlap ** k) * ((1.0 - overlap) ** (n_j - k)) * factorial(k)
                            for k in range(n_j + 1)], dtype=float)
        K = rng.choice(n_j + 1, p=weights / weights.sum())
        indist[j] = K
        dist[j] = n_j - K
    return indist, dist


def _sample_distinguishable(U128, particles, rng, reject):
    """sampling.py:403-418: every distinguishable photon lands in an output
    mode drawn from |U[:, input mode]|^2 (normalised), then may be lost."""
    d = len(particles)
    out = np.zeros(d, dtype=int)
    for mode, count in enumerate(particles):
        p = np.abs(U128[:, mode]) ** 2
        p = p / np.sum(p)
        for _ in range(count):
            o = rng.choice(d, p=p)
            if not reject():
                out[o] += 1
    return out


def _lockstep(U, U128, samples, photons, rngs, rejects):
    """The indistinguishable phase of every shot of a batch at once.  Shot s
    walks len(photons[s]) steps; at a step its reject flag (from the reject
    condition, in the reference's call order) either skips the step or it
    grows its input by a random remaining photon (its own generator), and all
    growing shots share ONE batched Laplace launch before each draws its
    output mode.  ``samples`` (shots x d) is updated in place."""
    nb, d = samples.shape
    current = np.zeros((nb, d), dtype=int)
    to_shrink = [list(p) for p in photons]
    steps = max((len(p) for p in photons), default=0)
    for k in range(steps):
        act = [s for s in range(nb) if k < len(photons[s]) and not rejects[s][k]]
        if not act:
            continue
        for s in act:
            i = rngs[s].choice(len(to_shrink[s]))
            current[s, to_shrink[s].pop(i)] += 1
        idx = np.asarray(act)
        lap = permanent_laplace_batch(U, samples[idx], current[idx]).astype(np.complex128)
        pmf = _pmf_batch(U128, current[idx], samples[idx], lap)
        u = np.array([rngs[s].random() for s in act])
        samples[idx, _draw_from_pmf(pmf, u)] += 1


def generate_samples(input_state, shots, interferometer, seed, batch_size=4096, transmission=None,
                     particle_overlap=None):
    """Samples of the reference's sampler, as tuples, in generation order.

    ``input_state``: occupation numbers (length d); ``interferometer``: the
    d x d matrix (its dtype picks complex64 or complex128 permanents);
    ``seed``: the reference's ``config.seed_sequence`` (shot idx uses seed + idx).
    ``transmission``: uniform loss — each photon step first asks the reject
    condition ``config.rng.uniform() > transmission`` of the configuration
    generator ``np.random.default_rng(seed)`` (passive/simulation_steps.py:
    351-362 of the reference), so shot s consumes that generator's draws
    s*n .. s*n+n-1.  ``particle_overlap``: uniform partial distinguishability
    (sampling.py:328-368): the photons of each shot are split into
    indistinguishable and distinguishable ones, the distinguishable ones are
    sampled one by one, the others by the exact sampler; the reject
    condition is asked once per photon in the same order.
    """
    U = np.asarray(interferometer)
    if U.dtype not in (np.complex64, np.complex128):
        U = U.astype(np.complex128)
    U128 = U.astype(np.complex128)
    inp = np.asarray(input_state).astype(int)
    d = len(inp)
    n = int(inp.sum())
    fq = to_first_quantized(inp)
    draws = None
    if transmission is not None:
        draws = np.random.default_rng(seed).uniform(size=shots * n) > transmission
    out = []
    for b0 in range(0, shots, batch_size):
        nb = min(batch_size, shots - b0)
        rngs = [np.random.default_rng(seed=seed + b0 + i) for i in range(nb)]
        samples = np.zeros((nb, d), dtype=int)    # the indistinguishable photons' outputs
        dist_out = np.zeros((nb, d), dtype=int)   # the distinguishable ones', added at the end
        photons, rejects = [], []
        for i in range(nb):
            flags = draws[(b0 + i) * n:(b0 + i + 1) * n] if draws is not None else np.zeros(n, dtype=bool)
            if particle_overlap is None:
                photons.append(fq)
                rejects.append(flags)
            else:
                indist, dist = _separate_particles(inp, particle_overlap, rngs[i])
                it = iter(flags[:int(dist.sum())])
                dist_out[i] = _sample_distinguishable(U128, dist, rngs[i], lambda: bool(next(it)))
                photons.append(to_first_quantized(indist))
                rejects.append(flags[int(dist.sum()):])
        _lockstep(U, U128, samples, photons, rngs, rejects)
        out.extend(tuple(int(x) for x in row) for row in samples + dist_out)
    return out


def expanded_interferometer(matrix):
    """The 2d x 2d dilation of a lossy d x d transmission matrix
    (sampling.py:756-784 of the reference): with the SVD M = V diag(s) W,
    blockdiag(V, I) [[diag s, diag c], [diag c, diag s]] blockdiag(W, I),
    c = sqrt(1 - s^2).  Its first d columns are orthonormal and its upper-left
    block is M; photons enter only the first d modes, so the lossless sampler
    on it samples the lossy channel.  numpy's SVD, as the reference's, fixes
    the phases (and so the samples of a given seed)."""
    M = np.asarray(matrix, dtype=np.complex128)
    V, sv, W = np.linalg.svd(M)
    d = len(sv)
    Z, I = np.zeros((d, d)), np.eye(d)
    c = np.diag(np.sqrt(np.maximum(0.0, 1.0 - sv ** 2)))
    return np.block([[V, Z], [Z, I]]) @ np.block([[np.diag(sv), c], [c, np.diag(sv)]]) @ np.block([[W, Z], [Z, I]])


def generate_lossy_samples(input_state, shots, matrix, seed, batch_size=4096, batched=False):
    """Non-uniform loss (sampling.py:110-146): the lossless sampler on the
    2d-mode dilation with d empty ancilla modes, samples trimmed to the first
    d modes.  ``batched``: the throughput sampler instead of the reference's
    per-seed sequence."""
    inp = np.asarray(input_state).astype(int)
    d = len(inp)
    E = expanded_interferometer(matrix)
    if np.asarray(matrix).dtype == np.complex64:
        E = E.astype(np.complex64)
    state = np.concatenate([inp, np.zeros(d, dtype=int)])
    if batched:
        return generate_samples_batched(state, shots, E, seed, batch_size=batch_size)[:, :d]
    return [s[:d] for s in generate_samples(state, shots, E, seed, batch_size=batch_size)]


def sample(input_state, shots, interferometer, seed, particle_overlap=None, batched=False, batch_size=4096,
           postselect=None):
    """The reference's dispatch (passive/simulation_steps.py:315-369): from the
    singular values of the interferometer, lossless (all 1), uniform loss
    (all equal: transmission s_0^2) or non-uniform loss (SVD dilation), with
    optional uniform particle overlap.  Non-uniform loss with partially
    distinguishable photons goes through loop hafnians in the reference and is
    not on this engine's path.

    ``postselect``: (modes, photon counts[, maximum trials per shot]), the
    reference's ``PostSelectPhotons`` before the measurement.  Samples then
    come from ``piquasso_gb300.postselect``: the reference's per-seed sequence
    with the shots' photon steps batched, or with ``batched`` rejection
    rounds of the throughput sampler (an int array)."""
    M = np.asarray(interferometer)
    sv = np.linalg.svd(M.astype(np.complex128), compute_uv=False)
    if postselect is not None:
        from . import postselect as ps

        if np.all(np.isclose(sv, sv[0])):
            T = None if np.isclose(sv[0], 1.0) else float(sv[0] ** 2)
            if batched:
                return ps.generate_samples_batched(input_state, shots, M, seed, postselect, transmission=T,
                                                   particle_overlap=particle_overlap, batch_size=batch_size)
            return ps.generate_samples(input_state, shots, M, seed, postselect, transmission=T,
                                       particle_overlap=particle_overlap)
        if particle_overlap is not None:
            raise NotImplementedError("non-uniform loss with partially distinguishable photons (loop hafnians)")
        if batched:
            return ps.generate_samples_batched(input_state, shots, M, seed, postselect, lossy=True,
                                               batch_size=batch_size)
        return ps.generate_lossy_samples(input_state, shots, M, seed, postselect)
    if np.all(np.isclose(sv, sv[0])):
        T = None if np.isclose(sv[0], 1.0) else float(sv[0] ** 2)
        if batched:
            return generate_samples_batched(input_state, shots, M, seed, batch_size=batch_size, transmission=T,
                                            particle_overlap=particle_overlap)
        return generate_samples(input_state, shots, M, seed, batch_size=batch_size, transmission=T,
                                particle_overlap=particle_overlap)
    if particle_overlap is not None:
        raise NotImplementedError("non-uniform loss with partially distinguishable photons (loop hafnians)")
    return generate_lossy_samples(input_state, shots, M, seed, batch_size=batch_size, batched=batched)


def is_direct_marginal_sampling_cheaper(k, d, n, shots):
    """The reference's rule for measuring k of d modes (sampling.py:860-887):
    direct marginal sampling when the marginal algorithm's coefficient count
    sum_{m<=n} C(m+k-1, k-1)^2 is small enough for the number of shots.  Kept
    as it is: the two methods draw different samples for a seed."""
    from math import comb

    if k == d:
        return False
    coeffs = sum(comb(m + k - 1, k - 1) ** 2 for m in range(n + 1))
    if coeffs <= 100_000:
        return True
    if coeffs <= 500_000:
        return shots >= 1_000
    if coeffs <= 4_000_000:
        return shots >= 10_000
    return False


def map_to_original_modes(modes, postselected_modes):
    """Active-mode indices (postselected modes removed) to the original
    numbering (sampling.py:787-793)."""
    m = np.asarray(modes, dtype=int).copy()
    for p in sorted(postselected_modes):
        m[m >= p] += 1
    return tuple(int(x) for x in m)


def measure(input_state, shots, interferometer, seed, modes=None, postselect=None, particle_overlap=None,
            batched=False):
    """``ParticleNumberMeasurement`` with shots, after an optional
    ``PostSelectPhotons`` (passive/simulation_steps.py:239-399): returns
    {outcome on ``modes``: count} in order of first occurrence.  ``modes``
    are numbered among the modes that survive the postselection (all of them
    by default).  A measurement of some of the modes with ideal or uniformly
    lossy optics samples the marginal directly when
    ``is_direct_marginal_sampling_cheaper`` says so (on the GPU marginals,
    ``marginals.generate_marginal_samples``; the reference takes this branch
    whatever the particle overlap); otherwise every mode is sampled
    (``sample``) and the outcomes are projected onto ``modes``."""
    from . import marginals

    inp = np.asarray(input_state).astype(int)
    d = len(inp)
    post_modes = tuple(int(m) for m in postselect[0]) if postselect else ()
    post_counts = tuple(int(c) for c in postselect[1]) if postselect else ()
    active = d - len(post_modes)
    modes = tuple(range(active)) if modes is None else tuple(int(m) for m in modes)
    marginal_only = set(modes) != set(range(active))
    M = np.asarray(interferometer)
    sv = np.linalg.svd(M.astype(np.complex128), compute_uv=False)
    n = int(inp.sum())
    if (marginal_only and np.all(np.isclose(sv, sv[0]))
            and is_direct_marginal_sampling_cheaper(len(modes) + len(post_modes), d, n, shots)):
        samples = marginals.generate_marginal_samples(inp, M, map_to_original_modes(modes, post_modes), shots, seed,
                                                      postselected_modes=post_modes,
                                                      postselected_photons=post_counts)
        return get_counts(samples)
    samples = sample(inp, shots, M, seed, particle_overlap=particle_overlap, batched=batched, postselect=postselect)
    if batched:
        samples = [tuple(int(x) for x in row) for row in samples]
    counts = get_counts(samples)
    if not marginal_only:
        return counts
    projected = {}
    for outcome, mult in counts.items():
        key = tuple(outcome[m] for m in modes)
        projected[key] = projected.get(key, 0) + mult
    return projected


def get_counts(samples):
    counts = {}
    for s in samples:
        counts[s] = counts.get(s, 0) + 1
    return counts


def result_samples(samples, seed):
    """What the reference's ``Result.samples`` returns for these samples."""
    out = []
    for outcome, mult in get_counts(samples).items():
        out.extend([tuple(outcome)] * mult)
    random.Random(seed).shuffle(out)
    return out


def generate_samples_batched(input_state, shots, interferometer, seed, batch_size=2048, timings=None,
                             transmission=None, particle_overlap=None, workers=2):
    """Exact samples of the same distribution, at throughput.

    Same algorithm (Clifford & Clifford B, sampling.py:208-236 of the
    reference): at step k a uniformly random not-yet-placed input photon joins
    the input, the conditional pmf over the d output modes comes from the
    Laplace permanents of (sample, current input), and one output mode is drawn.
    Differences from :func:`generate_samples`, all in the random-number
    plumbing: each batch of shots has its own generator
    ``np.random.default_rng((seed, batch))``, the photon order is a random
    permutation drawn up front (equivalent to picking a uniformly random
    remaining photon at every step), and the pmf and the draw are vectorised
    over shots.  The samples therefore follow the reference's distribution but
    not its per-seed sequence.  Batches run on ``workers`` threads, so one
    batch's host work (planning, pmf, draws) overlaps another's Laplace
    launches; the result does not depend on the thread count.  Returns an int
    array (shots, d).

    ``transmission`` (uniform loss): every photon is kept independently with
    this probability, so a shot samples a random subset of its photons — the
    distribution of the reference's per-step reject condition.
    ``particle_overlap``: each shot splits its photons as the reference's
    _separate_particles does; the distinguishable ones land independently
    (multinomial over |U[:, j]|^2), the rest go through the exact sampler.
    Shots with fewer photons left simply sit out the later steps.

    ``timings`` (optional dict) receives the seconds spent in the fused
    engine steps (Laplace permanents, pmf and draw: ``sampler_step_batch``)
    summed over the workers ("laplace_s") and the wall time ("total_s").
    """
    import time
    from concurrent.futures import ThreadPoolExecutor

    t_start = time.perf_counter()
    U = np.asarray(interferometer)
    if U.dtype not in (np.complex64, np.complex128):
        U = U.astype(np.complex128)
    U128 = U.astype(np.complex128)
    inp = np.asarray(input_state).astype(int)
    d = len(inp)
    n = int(inp.sum())
    colp = np.abs(U128) ** 2
    colp = colp / colp.sum(axis=0, keepdims=True)  # column j: landing probabilities of a photon from mode j
    fq = to_first_quantized(inp).astype(np.int64)
    rank = np.arange(n) - np.searchsorted(fq, fq)  # rank of each input photon among its mode's photons

    def one_batch(bi, nb):
        rng = np.random.default_rng((seed, bi))
        t_lap = 0.0
        rows = np.arange(nb)
        samples = np.zeros((nb, d), dtype=np.int64)    # the exact sampler's photons
        dist_out = np.zeros((nb, d), dtype=np.int64)   # distinguishable photons, added at the end
        # photon p of the input takes part in the exact sampler when it is
        # indistinguishable and kept
        take = np.ones((nb, n), dtype=bool)
        if particle_overlap is not None:
            from scipy.special import comb, factorial

            x = float(particle_overlap)
            K = np.zeros((nb, d), dtype=np.int64)
            for j in np.nonzero(inp)[0]:
                nj = int(inp[j])
                w = np.array([comb(nj, k) * x ** k * (1.0 - x) ** (nj - k) * factorial(k) for k in range(nj + 1)])
                K[:, j] = rng.choice(nj + 1, size=nb, p=w / w.sum())
            take = rank[None, :] < K[:, fq]
            dist = inp[None, :] - K
            if transmission is not None:
                dist = rng.binomial(dist, transmission)
            for j in np.nonzero(dist.sum(axis=0))[0]:
                dist_out += rng.multinomial(dist[:, j], colp[:, j])
        if transmission is not None:
            take &= rng.random((nb, n)) < transmission
        counts = take.sum(axis=1)
        m = int(counts.max()) if nb else 0
        # the photons of each shot in a uniformly random order (the others last)
        keys = rng.random((nb, n))
        keys[~take] = 2.0
        photons = fq[np.argsort(keys, axis=1)] if n else np.zeros((nb, 0), dtype=np.int64)
        current = np.zeros((nb, d), dtype=np.int64)
        for k in range(m):
            act = rows[counts > k]
            current[act, photons[act, k]] += 1
            first = samples[act].sum(axis=1) == 0
            u = rng.random(len(act))
            idx = np.zeros(len(act), dtype=np.int64)
            if np.any(~first):
                # Laplace permanents, pmf sum_j cur_j L_j U[idx, j] and draw:
                # one fused engine call, only the drawn modes come back
                t0 = time.perf_counter()
                sel = act[~first]
                idx[~first] = sampler_step_batch(U, samples[sel], current[sel], u[~first])
                t_lap += time.perf_counter() - t0
            if np.any(first):
                # empty output: the Laplace vector is [1] at the only input
                # column, so the pmf is |U[idx, j]|^2 of that column
                f = np.nonzero(first)[0]
                pmf = np.abs(U128[:, photons[act[f], k]].T) ** 2
                cdf = np.cumsum(pmf, axis=1)
                idx[f] = np.minimum((cdf < (u[f] * cdf[:, -1])[:, None]).sum(axis=1), d - 1)
            samples[act, idx] += 1
        return samples + dist_out, t_lap

    batches = [(bi, min(batch_size, shots - b0)) for bi, b0 in enumerate(range(0, shots, batch_size))]
    out = np.zeros((shots, d), dtype=np.int64)
    t_lap = 0.0
    with ThreadPoolExecutor(max_workers=max(1, int(workers))) as ex:
        for (bi, nb), (S, tl) in zip(batches, ex.map(lambda a: one_batch(*a), batches)):
            out[bi * batch_size:bi * batch_size + nb] = S
            t_lap += tl
    if timings is not None:
        timings["laplace_s"] = t_lap
        timings["total_s"] = time.perf_counter() - t_start
    return out
