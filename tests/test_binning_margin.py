"""CPU check of the count pass's scaled-guess binning (guess_bin in k_hist, k_bisect_tile and
k_subtree): whenever the guess is accepted by the margin test it is the exact leaf of the
midpoint tree, i.e. the bin the reference's bisection descent reaches. float32 restatement of
the device arithmetic, the fused multiply-add y = fl(fl(k-L) scale + 2^11) rounded once (exact
products in float64, rational arithmetic where the float64 sum is inexact); the margin here
uses round-to-nearest (the device rounds it up), so it accepts at least as many guesses as
the device does."""
from fractions import Fraction

import numpy as np

f32 = np.float32


def midpoint_edges(L, R, K):
    """Edge table e[0..2^K] of the midpoint tree over [L, R] (float32 midpoints, in order)."""
    nb = 1 << K
    e = np.empty(nb + 1, f32)
    e[0], e[nb] = L, R
    for d in range(K):
        s = nb >> (d + 1)
        j = np.arange(s, nb, 2 * s)
        e[j] = (e[j + s] + e[j - s]) * f32(0.5)  # mid_cut: fl(fl(R + L) * 0.5)
    return e


def margin(L, R, scale, nb):
    M = max(abs(L), abs(R))
    e = int(np.array(M, f32).view(np.uint32)) >> 23 & 0xFF
    if e < 24 or e == 0xFF:
        return f32(1.0)
    u = np.array((e - 23) << 23, np.uint32).view(f32)[()]
    return f32(f32(f32(8.0) * u) * scale) + f32(f32(nb) * f32(2.0 ** -21))


def _round_f32(q: Fraction) -> np.float32:
    """q rounded to the nearest float32, ties to even (q inside the float32 range)."""
    c = f32(float(q))
    best = None
    for cand in (np.nextafter(c, f32(-np.inf)), c, np.nextafter(c, f32(np.inf))):
        dist = abs(Fraction(float(cand)) - q)
        key = (dist, int(np.array(cand, f32).view(np.uint32)) & 1)
        if best is None or key < best[0]:
            best = (key, cand)
    return f32(best[1])


def fma_2048(a, scale):
    """float32 fl(a * scale + 2048) rounded once, for float32 arrays a and scalar scale."""
    p = a.astype(np.float64) * np.float64(scale)  # exact: 24 x 24 bits
    s = p + 2048.0
    y = s.astype(f32)
    inexact = np.isfinite(p) & ((s - 2048.0) != p)
    for i in np.nonzero(inexact)[0]:
        y[i] = _round_f32(Fraction(float(a[i])) * Fraction(float(scale)) + 2048)
    return y


def guess_bin(k, L, R, scale, nb):
    """(ok, bin) of the device's guess_bin over keys k."""
    M = f32(margin(L, R, scale, max(nb, 2048)) * f32(4096.0))
    if M < 2048:
        mi = int(M)
        span = 4095 - 2 * mi
    else:
        mi, span = 0, 0
    base = int(np.array(2048.0, f32).view(np.uint32)) + mi + 1
    y = fma_2048((k - f32(L)).astype(f32), scale)
    e = (y.view(np.uint32).astype(np.int64) - base) & 0xFFFFFFFF
    ok = (e < (nb << 12)) & ((e & 0xFFF) < span)
    return ok, e >> 12


def check_bracket(rng, L, R, K, nkeys):
    nb = 1 << K
    e = midpoint_edges(L, R, K)
    scale = f32(nb) / f32(R - L)
    # keys: uniform in [L, R), plus edges and their float neighbours
    k = (f32(L) + f32(R - L) * rng.random(nkeys).astype(f32)).astype(f32)
    j = rng.integers(0, nb + 1, nkeys // 4)
    near = np.concatenate([e[j], np.nextafter(e[j], f32(np.inf)), np.nextafter(e[j], f32(-np.inf))])
    k = np.concatenate([k, near.astype(f32)])
    k = k[(k >= L) & (k < R)]
    exact = np.searchsorted(e[:nb], k, side="right") - 1  # largest b with e[b] <= k
    ok, g = guess_bin(k, L, R, scale, nb)
    bad = ok & (g != exact)
    # keys outside [L, R) (neighbours of the end edges, NaN) are never accepted
    out = np.concatenate([np.nextafter(np.array([L, L], f32), f32(-np.inf)), np.array([R], f32),
                          np.nextafter(np.array([R], f32), f32(np.inf)),
                          np.array([np.nan, np.inf, -np.inf], f32)])
    ok_out, _ = guess_bin(out, L, R, scale, nb)
    assert not ok_out.any(), f"key outside [{L!r}, {R!r}) accepted"
    return int(ok.sum()), int(bad.sum()), len(k)


def test_accepted_guesses_are_exact():
    rng = np.random.default_rng(5)
    accepted = total = 0
    for trial in range(400):
        K = int(rng.integers(4, 12))
        mode = trial % 4
        if mode == 0:  # boxes of the unit cube and their sub-brackets
            L = f32(-0.5 + (rng.integers(0, 1 << 24) * 2.0 ** -24))
            R = f32(L + f32(2.0 ** -int(rng.integers(0, 20))))
        elif mode == 1:  # anywhere, any width
            L = f32(rng.uniform(-1e3, 1e3))
            R = f32(L + f32(10.0 ** rng.uniform(-5, 2)))
        elif mode == 2:  # a few hundred ulps wide
            L = f32(rng.uniform(-1, 1))
            R = L
            for _ in range(int(rng.integers(1, 400))):
                R = np.nextafter(R, f32(np.inf))
        else:  # straddling zero
            w = f32(10.0 ** rng.uniform(-6, 0))
            L = f32(-w * f32(rng.random()))
            R = f32(L + w)
        if not (L < R) or not np.isfinite(R - L):
            continue
        a, bad, n = check_bracket(rng, L, R, K, 4000)
        assert bad == 0, f"guess off its exact bin in [{L!r}, {R!r}) K={K}"
        accepted += a
        total += n
    assert accepted > 0


def test_guess_settles_almost_every_key_of_a_box():
    # the first pass of the unit box: uniform keys, 2048 bins
    rng = np.random.default_rng(6)
    L, R, K = f32(-0.5), f32(0.5), 11
    nb = 1 << K
    scale = f32(nb) / f32(R - L)
    k = (L + f32(R - L) * rng.random(200000).astype(f32)).astype(f32)
    ok, _ = guess_bin(k, L, R, scale, nb)
    assert ok.mean() > 0.99


def near_bin(k, L, scale, e, top):
    """Restatement of the device's near_bin for keys L <= k < R: the floor of the same guess
    (its fused multiply-add encoding, clamped to the top leaf), then the guessed leaf or a
    neighbour checked against the edge table; None where the device falls back to a search."""
    y = fma_2048((k - f32(L)).astype(f32), scale)
    t = y.view(np.uint32).astype(np.int64) - 0x45000000  # the encoding of 2048.0f
    g = np.minimum(t >> 12, top)
    res = np.full(k.shape, -1, np.int64)
    below = k < e[g]
    inside = ~below & (k < e[g + 1])
    res[inside] = g[inside]
    lo = below & (g > 0)
    lo_ok = lo.copy()
    lo_ok[lo] = ~(k[lo] < e[g[lo] - 1])
    res[lo_ok] = g[lo_ok] - 1
    hi = ~below & ~inside & (g < top)
    hi_ok = hi.copy()
    hi_ok[hi] = k[hi] < e[g[hi] + 2]
    res[hi_ok] = g[hi_ok] + 1
    return res  # -1: the search


def test_rejected_keys_need_no_search_when_the_guess_is_trusted():
    """The exact path of the count pass (near_bin): where the margin lets the guess be trusted
    (its bins are more than 16 ulps wide) the guessed leaf or a neighbour is the exact leaf,
    so the edge-table search is never taken; every bin it returns is the exact one."""
    rng = np.random.default_rng(7)
    checked = 0
    for trial in range(300):
        K = int(rng.integers(4, 12))
        nb = 1 << K
        if trial % 2 == 0:
            L = f32(-0.5 + (rng.integers(0, 1 << 24) * 2.0 ** -24))
            R = f32(L + f32(2.0 ** -int(rng.integers(0, 20))))
        else:
            L = f32(rng.uniform(-1e3, 1e3))
            R = f32(L + f32(10.0 ** rng.uniform(-5, 2)))
        if not (L < R) or not np.isfinite(R - L):
            continue
        e = midpoint_edges(L, R, K)
        scale = f32(nb) / f32(R - L)
        k = (f32(L) + f32(R - L) * rng.random(3000).astype(f32)).astype(f32)
        j = rng.integers(0, nb + 1, 1000)
        near = np.concatenate([e[j], np.nextafter(e[j], f32(np.inf)), np.nextafter(e[j], f32(-np.inf))])
        k = np.concatenate([k, near.astype(f32)])
        k = k[(k >= L) & (k < R)]
        exact = np.searchsorted(e[:nb], k, side="right") - 1
        got = near_bin(k, L, scale, e, nb - 1)
        found = got >= 0
        assert np.array_equal(got[found], exact[found]), f"near_bin off in [{L!r}, {R!r}) K={K}"
        trusted = f32(margin(L, R, scale, max(nb, 2048)) * f32(4096.0)) < 2048
        if trusted:
            assert found.all(), f"search needed in a trusted bracket [{L!r}, {R!r}) K={K}"
            checked += 1
    assert checked > 50
