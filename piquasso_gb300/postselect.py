"""Postselected exact boson sampling (``PostSelectPhotons`` followed by
``ParticleNumberMeasurement`` in the reference).

The reference's samplers with ``postselect_data`` (piquasso/_simulators/
passive/sampling.py:239-326 and :422-643) retry each shot until the photons
counted in the postselected modes equal the requested numbers:

* indistinguishable photons (``_generate_sample_with_postselect``): a trial
  is the Clifford & Clifford walk of one shot, abandoned as soon as a
  postselected mode holds too many photons, or as soon as the photons still
  needed there exceed the photons still to place;
* partially distinguishable photons (``_generate_sample_with_postselect_and_uniform_overlap``):
  a trial splits the photons, runs ONE trial of the walk above for the
  indistinguishable ones, accepts the rest with the probability that the
  distinguishable photons complete the postselected counts (a truncated
  generating polynomial), then samples them conditioned on that (a table of
  completion probabilities, one per remaining photon).

Each shot follows the reference's random-number sequence exactly, with its own
``np.random.default_rng(seed + idx)`` and the shared configuration generator
for uniform loss, so a seed reproduces the reference's samples.  Each shot is
written as a generator. Its photon steps yield (input so far, output so far)
and receive the step's pmf. ``_drive`` answers every shot waiting on a step
with one batched Laplace-permanent launch (``permanent_laplace_batch``).
Shots run side by side unless a uniform-loss reject condition draws from
the shared generator. Then they run one after another, because the number of
draws a shot takes depends on its trials.

The reference divides the postselected output by deleting the postselected
modes (``np.delete``). For non-uniform loss it does this on the 2d-mode dilated
sample and then keeps its first d entries (sampling.py:110-146). Both are
kept as they are.
"""

import numpy as np

from .permanent import permanent_laplace_batch
from .sampling import _draw_from_pmf, _pmf_batch, _separate_particles, expanded_interferometer, to_first_quantized


class InvalidSimulation(RuntimeError):
    """A shot used up its trials (the reference's
    ``piquasso.api.exceptions.InvalidSimulation``, same message)."""


DEFAULT_MAX_TRIALS = 1000  # Config.max_sample_generation_trials (piquasso/api/config.py:78)


def _trial_limit(limit):
    return InvalidSimulation(
        "Too many trials during sample generation. "
        "The specified postselection criteria may be very highly unlikely. "
        "Aborting. "
        "To increase the limit, set Config.max_sample_generation_trials "
        f"to a higher value. Current value: {limit}.")


def _shot(d, n, photons, rng, reject, modes, counts, max_trials, track_needed=True):
    """One shot of sampling.py:239-326 as a generator: for each photon step it
    yields (input, output, its generator) and receives the mode drawn from the
    step's pmf with that generator.  Returns the output with the
    postselected modes deleted, or the whole output when ``track_needed`` is
    False (the partially distinguishable sampler's inner call)."""
    modes = tuple(int(m) for m in modes)
    needed0 = np.sum(counts)
    current = np.empty(d, dtype=int)
    sample = np.empty(d, dtype=int)
    trial = 0
    while True:
        trial += 1
        if trial > max_trials:
            raise _trial_limit(max_trials)
        current[:] = 0
        sample[:] = 0
        needed = needed0
        left = np.array(counts, dtype=int)  # photons each postselected mode may still take
        pool = list(photons)
        complete = True
        for k in range(1, n + 1):
            if reject():
                continue
            i = rng.choice(len(pool))
            current[pool.pop(i)] += 1
            mode = yield current, sample, rng
            sample[mode] += 1
            if mode in modes:
                needed -= 1
                left[modes.index(mode)] -= 1
                if np.any(left < 0):
                    complete = False
                    break
            if track_needed and needed > n - k:
                complete = False
                break
        if complete:
            break
    if not track_needed:
        return sample.copy()
    return np.delete(sample, modes)


def _times_linear(poly, constant, coeffs, out):
    """out = (constant + sum_j coeffs[j] x_j) * poly, truncated to poly's
    shape (the reference's multiply_by_linear_truncated,
    piquasso/_math/polynomial.py:19-40, same operations in the same order).
    With ``out is poly`` each axis's term reads the array already updated by
    the constant and the earlier axes, so the product becomes
    constant * prod_j (1 + coeffs[j] x_j) * poly. The reference's acceptance
    probability calls it this way (sampling.py:545-549), and the samples of a
    seed depend on it."""
    out[...] = constant * poly
    for axis, c in enumerate(coeffs):
        hi = [slice(None)] * poly.ndim
        lo = list(hi)
        hi[axis] = slice(1, None)
        lo[axis] = slice(None, -1)
        out[tuple(hi)] += c * poly[tuple(lo)]
    return out


def _real_dtype(U):
    return np.finfo(U.dtype).dtype


def _acceptance(U, dist, modes, counts):
    """sampling.py:533-551: the coefficient of x^counts in the product, over
    the distinguishable photons, of (stay-out probability + sum_j p_j x_j),
    p_j = |U[mode j, input]|^2 (multiplied in place)."""
    poly = np.zeros(tuple(np.asarray(counts) + 1), dtype=_real_dtype(U))
    poly[(0,) * len(counts)] = 1.0
    for j, m in enumerate(dist):
        p = np.abs(U[modes, j]) ** 2
        for _ in range(m):
            _times_linear(poly, 1.0 - p.sum(), p, out=poly)
    return poly[tuple(counts)]


def _completion_tables(U, dist, modes, bound):
    """sampling.py:554-583: table[i][c] = the probability that photons i, i+1,
    ... of the distinguishable input (first quantized) put exactly c photons
    into the postselected modes."""
    fq = to_first_quantized(dist)
    tables = [np.zeros(tuple(np.asarray(bound) + 1), dtype=_real_dtype(U)) for _ in range(len(fq) + 1)]
    tables[-1][(0,) * len(bound)] = 1.0
    for i in range(len(fq) - 1, -1, -1):
        p = np.abs(U[modes, fq[i]]) ** 2
        _times_linear(tables[i + 1], 1.0 - p.sum(), p, out=tables[i])
    return tables


def _conditioned_outputs(U, dist, modes, counts, tables, rng):
    """sampling.py:586-643: each distinguishable photon in turn lands in a
    free mode, is lost, or lands in a postselected mode that still needs a
    photon, weighted by the probability that the photons after it complete
    the counts; one ``rng.choice`` per photon over [free modes, loss,
    postselected modes].  The loss weight 1 - sum |U[:, j]|^2 is clamped at
    zero: for a unitary it can round to about -1e-16, which the reference
    passes to ``rng.choice`` and which numpy rejects."""
    d = U.shape[0]
    fq = to_first_quantized(dist)
    free = np.delete(np.arange(d), modes)
    out = np.zeros(d, dtype=int)
    left = np.array(counts, dtype=int)
    for i, j in enumerate(fq):
        nxt = tables[i + 1]
        future = nxt[tuple(left)]
        p_free = np.abs(U[free, j]) ** 2
        p_sel = np.abs(U[modes, j]) ** 2
        loss = 1.0 - p_free.sum() - p_sel.sum()
        if loss < 0:
            loss = np.zeros_like(loss)
        w_sel = np.zeros(len(modes), dtype=_real_dtype(U))
        for a, p in enumerate(p_sel):
            if left[a] == 0:
                continue
            left[a] -= 1
            w_sel[a] = p * nxt[tuple(left)]
            left[a] += 1
        w = np.concatenate([p_free * future, np.array([loss * future], dtype=_real_dtype(U)), w_sel])
        w /= np.sum(w)
        k = rng.choice(len(w), p=w)
        if k < len(free):
            out[free[k]] += 1
        elif k > len(free):
            a = k - len(free) - 1
            out[modes[a]] += 1
            left[a] -= 1
    return out


def _overlap_shot(d, U, inp, rng, reject, modes, counts, max_trials, overlap):
    """One shot of sampling.py:422-530 as a generator."""
    modes = np.asarray(modes, dtype=int)
    counts = np.asarray(counts, dtype=int)
    trial = 0
    while True:
        trial += 1
        if trial > max_trials:
            raise _trial_limit(max_trials)
        indist, dist = _separate_particles(inp, overlap, rng)
        try:
            indist_out = yield from _shot(d, np.sum(indist), to_first_quantized(indist), rng, reject, modes,
                                          counts, 1, track_needed=False)
        except InvalidSimulation:
            continue
        left = counts - indist_out[modes]
        if rng.random() > _acceptance(U, dist, modes, left):
            continue
        tables = _completion_tables(U, dist, modes, counts)
        out = _conditioned_outputs(U, dist, modes, left, tables, rng) + indist_out
        return np.delete(out, modes)


def _drive(U, shots, side_by_side):
    """Runs the shot generators.  Every shot waiting on a photon step gets its
    pmf from one batched Laplace launch over all of them (the pmf as the
    reference's _calculate_pmf forms it, sampling.py:723-749) and its mode
    from one ``random()`` of its own generator (what ``rng.choice`` with p
    draws, sampling.py:752-753).  With ``side_by_side`` False the shots run
    one after another."""
    U128 = U.astype(np.complex128)
    results = [None] * len(shots)
    groups = [list(range(len(shots)))] if side_by_side else [[i] for i in range(len(shots))]
    for group in groups:
        waiting = {}

        def advance(i, pmf):
            try:
                waiting[i] = shots[i].send(pmf)
            except StopIteration as stop:
                results[i] = stop.value

        for i in group:
            advance(i, None)
        while waiting:
            idx = list(waiting)
            cols = np.stack([waiting[i][0] for i in idx])
            rows = np.stack([waiting[i][1] for i in idx])
            gens = [waiting[i][2] for i in idx]
            waiting.clear()
            lap = permanent_laplace_batch(U, rows, cols).astype(np.complex128)
            pmf = _pmf_batch(U128, cols, rows, lap)
            modes = _draw_from_pmf(pmf, np.array([g.random() for g in gens]))
            for r, i in enumerate(idx):
                advance(i, int(modes[r]))
    return results


def generate_samples(input_state, shots, interferometer, seed, postselect, transmission=None,
                     particle_overlap=None):
    """Postselected samples as the reference's ``generate_samples`` makes them
    with ``postselect_data`` (sampling.py:33-102), as tuples in shot order.

    ``postselect``: (modes, photon counts) or (modes, photon counts, maximum
    trials per shot; default 1000, the reference's
    Config.max_sample_generation_trials).  ``transmission``: uniform loss,
    ``config.rng.uniform() > transmission`` per photon step from
    ``np.random.default_rng(seed)`` (passive/simulation_steps.py:351-362).
    ``particle_overlap``: uniform partial distinguishability.  The postselected
    modes are deleted from every sample.  Raises ``InvalidSimulation`` when a
    shot uses up its trials."""
    modes, counts = tuple(int(m) for m in postselect[0]), tuple(int(c) for c in postselect[1])
    max_trials = int(postselect[2]) if len(postselect) > 2 else DEFAULT_MAX_TRIALS
    if len(modes) != len(counts) or len(set(modes)) != len(modes):
        raise ValueError("postselect needs one photon count per distinct mode")
    U = np.asarray(interferometer)
    if U.dtype not in (np.complex64, np.complex128):
        U = U.astype(np.complex128)
    inp = np.asarray(input_state).astype(int)
    d = len(inp)
    if any(m < 0 or m >= d for m in modes) or any(c < 0 for c in counts):
        raise ValueError("postselected modes must lie in 0..d-1 with nonnegative counts")
    n = np.sum(inp)
    if transmission is None:
        reject = lambda: False  # noqa: E731
    else:
        cfg = np.random.default_rng(seed)
        reject = lambda: cfg.uniform() > transmission  # noqa: E731
    gens = []
    for idx in range(shots):
        rng = np.random.default_rng(seed=seed + idx)
        if particle_overlap is None:
            gens.append(_shot(d, n, to_first_quantized(inp), rng, reject, modes, counts, max_trials))
        else:
            gens.append(_overlap_shot(d, U, inp, rng, reject, modes, counts, max_trials, particle_overlap))
    return [tuple(int(x) for x in s) for s in _drive(U, gens, side_by_side=transmission is None)]


def generate_lossy_samples(input_state, shots, matrix, seed, postselect):
    """Non-uniform loss with postselection (sampling.py:105-146): the
    postselected sampler on the 2d-mode dilation with d empty ancilla modes;
    each sample, its postselected modes already deleted, is cut to its first
    d entries."""
    inp = np.asarray(input_state).astype(int)
    d = len(inp)
    E = expanded_interferometer(matrix)
    if np.asarray(matrix).dtype == np.complex64:
        E = E.astype(np.complex64)
    state = np.concatenate([inp, np.zeros(d, dtype=int)])
    return [s[:d] for s in generate_samples(state, shots, E, seed, postselect)]


def _round_seed(seed, r):
    """An independent 63-bit seed for round r of a rejection loop."""
    return int(np.random.SeedSequence([int(seed), int(r)]).generate_state(1, dtype=np.uint64)[0] >> np.uint64(1))


def generate_samples_batched(input_state, shots, interferometer, seed, postselect, transmission=None,
                             particle_overlap=None, lossy=False, batch_size=2048):
    """Postselected samples at throughput: rounds of unconditioned samples
    from ``sampling.generate_samples_batched`` (one fused Laplace + pmf + draw
    launch per photon step for all shots of a batch), keeping the samples
    whose postselected modes hold exactly the requested counts.  Those follow
    the conditional distribution that the reference's retry loop samples, but
    not its per-seed sequence.  ``lossy``: non-uniform loss, sampled on the
    2d-mode dilation and trimmed as the reference trims it (postselected
    modes deleted, then the first d entries).  Raises ``InvalidSimulation``
    after (maximum trials) x shots samples without enough matches.  Returns
    an int array (shots, remaining modes)."""
    from . import sampling

    modes, counts = tuple(int(m) for m in postselect[0]), np.array([int(c) for c in postselect[1]], dtype=int)
    max_trials = int(postselect[2]) if len(postselect) > 2 else DEFAULT_MAX_TRIALS
    M = np.asarray(interferometer)
    inp = np.asarray(input_state).astype(int)
    d = len(inp)
    if lossy:
        E = expanded_interferometer(M)
        if M.dtype == np.complex64:
            E = E.astype(np.complex64)
        M, inp = E, np.concatenate([inp, np.zeros(d, dtype=int)])
    D = len(inp)
    if len(modes) != len(counts) or len(set(modes)) != len(modes) or any(m < 0 or m >= D for m in modes) \
            or np.any(counts < 0):
        raise ValueError("postselect needs one nonnegative photon count per distinct mode in 0..d-1")
    kept, have, drawn, r = [], 0, 0, 0
    while have < shots:
        if drawn >= max_trials * shots:
            raise _trial_limit(max_trials)
        rate = max(have / drawn, 1.0 / max_trials) if drawn else 1.0
        k = int(min(max(batch_size, np.ceil(1.2 * (shots - have) / rate)), max_trials * shots - drawn, 1 << 20))
        S = sampling.generate_samples_batched(inp, k, M, _round_seed(seed, r), batch_size=batch_size,
                                              transmission=transmission, particle_overlap=particle_overlap)
        drawn += k
        r += 1
        ok = np.all(S[:, list(modes)] == counts, axis=1)
        out = np.delete(S[ok], list(modes), axis=1)
        kept.append(out[:, :d] if lossy else out)
        have += len(out)
    if not kept:
        return np.zeros((0, min(d, D - len(modes)) if lossy else D - len(modes)), dtype=int)
    return np.concatenate(kept)[:shots]
