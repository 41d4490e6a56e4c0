"""The double-float walk's exact column sums, restated in numpy (no GPU).

The prep kernel rounds every scaled matrix entry to a multiple of 2^-47
(prep.cuh, q47) and splits seeds, update rows and prefix-table entries with
their high words on the grid of multiples of 2^-23 (walk_df.cuh,
df_split_grid).  The walk then forms column sums as hi + hi, lo + lo and a
Fast2Sum (df_grid_sum), and moves seeds by df_grid_add.  These tests check,
on random values in the ranges the column scaling guarantees (sums below 1,
table entries and update rows below 2), that every one of those FP32
operations is exact, i.e. that the claims the kernels rely on hold for IEEE
binary32 round-to-nearest arithmetic.
"""

import numpy as np

F = np.float32
Q47 = 2.0 ** 47
GRID = F(2.0 ** -23)


def q47(x):
    return np.rint(x * Q47) / Q47


def split_grid(x):
    """df_split_grid: high word on the 2^-23 grid, the rest as a float."""
    hi = (np.rint(x * 2.0 ** 23) * 2.0 ** -23).astype(F)
    lo = (x - hi.astype(np.float64)).astype(F)
    return hi, lo


def grid_sum(ah, al, bh, bl):
    """df_grid_sum: exact high and low sums, then Fast2Sum."""
    h = ah + bh
    l_ = al + bl
    s = h + l_
    return s, l_ - (s - h), h, l_


def grid_add(ah, al, bh, bl):
    """df_grid_add: exact sums, the low word's grid part moved into the high word."""
    h = ah + bh
    l_ = al + bl
    t = (l_ + F(1.5)) - F(1.5)
    return h + t, l_ - t


def _entries(rng, n, bound):
    """Sums of scaled, rounded matrix entries below `bound` in magnitude."""
    k = rng.integers(1, 30, size=n)
    x = np.zeros(n)
    for i in range(n):
        parts = q47(rng.uniform(-1.0, 1.0, size=k[i]) * (bound / k[i]) * 0.999)
        x[i] = parts.sum()  # exact in FP64: multiples of 2^-47 below 2
    return x


def test_split_is_exact():
    rng = np.random.default_rng(1)
    for bound in (1.0, 2.0):
        x = _entries(rng, 20000, bound)
        hi, lo = split_grid(x)
        assert np.all(hi.astype(np.float64) + lo.astype(np.float64) == x)
        assert np.all(np.abs(lo) <= 2.0 ** -24)
        assert np.all(np.rint(hi.astype(np.float64) * 2.0 ** 23) == hi.astype(np.float64) * 2.0 ** 23)


def test_column_sum_is_exact_and_normalised():
    rng = np.random.default_rng(2)
    seed = _entries(rng, 20000, 1.0)
    delta = _entries(rng, 20000, 2.0)
    keep = np.abs(seed + delta) < 1.0  # the column scaling's guarantee for a column sum
    seed, delta = seed[keep], delta[keep]
    sh, sl = split_grid(seed)
    dh, dl = split_grid(delta)
    s, lo, h, l_ = grid_sum(sh, sl, dh, dl)
    exact = seed + delta
    # hi + hi and lo + lo are exact
    assert np.all(h.astype(np.float64) == sh.astype(np.float64) + dh.astype(np.float64))
    assert np.all(l_.astype(np.float64) == sl.astype(np.float64) + dl.astype(np.float64))
    # the renormalised pair represents the exact sum, with a low word below half an ulp
    assert np.all(s.astype(np.float64) + lo.astype(np.float64) == exact)
    ulp = np.spacing(np.abs(s)).astype(np.float64)
    assert np.all(np.abs(lo.astype(np.float64)) <= ulp / 2)


def test_seed_update_stays_exact_on_the_grid():
    rng = np.random.default_rng(3)
    seed = _entries(rng, 5000, 0.5)
    sh, sl = split_grid(seed)
    val = seed.copy()
    for _ in range(200):  # a walk of one-digit updates
        d = _entries(rng, 5000, 0.05) * 2.0
        d = np.where(np.abs(val + d) < 1.0, d, -d)
        dh, dl = split_grid(d)
        sh, sl = grid_add(sh, sl, dh, dl)
        val = val + d  # exact in FP64
        assert np.all(sh.astype(np.float64) + sl.astype(np.float64) == val)
        assert np.all(np.abs(sl) <= 2.0 ** -24)


def test_regrid_of_a_double_float_seed_is_exact():
    """df_to_grid: a standard double-float (hi, lo) of a value on the 2^-47 grid
    below 1 moves onto the grid without rounding (hi - t exact, then one add,
    then the low word's grid part into the high word)."""
    rng = np.random.default_rng(4)
    x = _entries(rng, 20000, 1.0)
    hi = x.astype(F)
    lo = (x - hi.astype(np.float64)).astype(F)
    assert np.all(hi.astype(np.float64) + lo.astype(np.float64) == x)
    t = (np.rint(hi * F(2.0 ** 23)) * GRID).astype(F)
    l_ = (hi - t) + lo
    assert np.all(t.astype(np.float64) + l_.astype(np.float64) == x)  # exact, but |l_| up to 1.5 * 2^-24
    u = (l_ + F(1.5)) - F(1.5)
    nhi, nlo = t + u, l_ - u
    assert np.all(nhi.astype(np.float64) + nlo.astype(np.float64) == x)
    assert np.all(np.abs(nlo) <= 2.0 ** -24)
    # and the regridded seed's column sums stay exact
    delta = _entries(rng, 20000, 1.0)
    keep = np.abs(x + delta) < 1.0
    dh, dl = split_grid(delta[keep])
    s, lo2, h, l2 = grid_sum(nhi[keep], nlo[keep], dh, dl)
    assert np.all(s.astype(np.float64) + lo2.astype(np.float64) == x[keep] + delta[keep])
