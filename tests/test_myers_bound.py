"""The lower bound the head pass of GPU verification stops candidates on (CPU).

After the first 64 read bases the head pass takes the minimum of the band
cells the reference's final scan would look at (cells 0 .. last_high: the site
error plus the running sum of the VP / VN bits, mapper_cpe.c:634-650) and,
when it is above e, writes (10000, -1) without running the remaining bases.
That is exact only if no cell of a later step falls below that minimum. These
tests run the reference's banded Myers recurrence (banded_myers_simd,
mapper_cpe.c:519-660) vectorised over many candidates, pin it to the oracle's
restatement bit for bit, and check the bound at every step on random,
mutated, low-complexity and periodic windows for every threshold e <= 15.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po

MAXERROR = 10000


def _cases(rng, n, L, e, rl):
    """Windows of rl + 32 bases and reads of L bases: a mix of unrelated
    reads, copies of the window at 2-20% divergence (substitutions and
    1-base indels) from a random band offset, and 2-letter / periodic
    sequences."""
    win = rng.integers(0, 4, (n, rl + 32), dtype=np.uint8)
    kind = rng.integers(0, 6, n)
    low = kind >= 4
    win[low] &= 1
    per = kind == 5
    period = rng.integers(1, 7, n)
    idx = np.arange(rl + 32)
    win[per] = (idx[None, :] % period[per, None]).astype(np.uint8) & 3
    rd = rng.integers(0, 4, (n, L), dtype=np.uint8)
    div = np.choose(np.minimum(kind, 4), [1.0, 0.02, 0.08, 0.2, 0.1])
    for c in np.nonzero(kind > 0)[0]:
        wi = int(rng.integers(0, 2 * e + 1))
        for i in range(L):
            u = rng.random()
            d = div[c]
            src = win[c, min(wi, rl + 31)]
            if u < 0.7 * d:
                rd[c, i] = (src + rng.integers(1, 4)) & 3
                wi += 1
            elif u < 0.85 * d:
                rd[c, i] = rng.integers(0, 4)
            elif u < d:
                wi += 1
                rd[c, i] = win[c, min(wi, rl + 31)]
                wi += 1
            else:
                rd[c, i] = src
                wi += 1
    return win, rd


def _myers(win, rd, e, rl):
    """The recurrence over all cases at once: returns the final (error, loc)
    per case and, per case, the largest scan-range minimum seen at any step
    minus the smallest final-scan cell (must be <= 0)."""
    n, L = rd.shape
    W = 2 * e + 1
    mask = np.uint32((1 << W) - 1)
    lh = rl - L
    vp = np.zeros(n, np.uint32)
    vn = np.zeros(n, np.uint32)
    err = np.zeros(n, np.int64)
    worst = np.full(n, -10**9, np.int64)
    mins = []
    for i in range(L):
        eq = np.zeros(n, np.uint32)
        for j in range(W):
            eq |= (win[:, i + j] == rd[:, i]).astype(np.uint32) << np.uint32(j)
        eq &= mask
        x = eq | vn
        d0 = ((vp + (x & vp)) ^ vp) | x
        hn = vp & d0
        hp = vn | ~(vp | d0)
        x = d0 >> np.uint32(1)
        vn = x & hp
        vp = hn | ~(x | hp)
        err += ((d0 & np.uint32(1)) == 0)
        c = err.copy()
        m = err.copy()
        for k in range(lh):
            c += ((vp >> np.uint32(k)) & np.uint32(1)).astype(np.int64)
            c -= ((vn >> np.uint32(k)) & np.uint32(1)).astype(np.int64)
            np.minimum(m, c, out=m)
        mins.append(m)
    # final scan: first strict minimum <= e
    error = np.full(n, MAXERROR, np.int64)
    loc = np.full(n, -1, np.int64)
    c = err.copy()
    fmin = c.copy()
    hit = (c <= e)
    error[hit] = c[hit]
    loc[hit] = L - 1
    for k in range(lh):
        c += ((vp >> np.uint32(k)) & np.uint32(1)).astype(np.int64)
        c -= ((vn >> np.uint32(k)) & np.uint32(1)).astype(np.int64)
        np.minimum(fmin, c, out=fmin)
        better = (c <= e) & (c < error)
        error[better] = c[better]
        loc[better] = L + k
    for m in mins:
        np.maximum(worst, m - fmin, out=worst)
    return error, loc, worst, mins


def _oracle_myers(win, rd, e, rl):
    """swo_banded_myers on one case: w2 the 2-bit packed read, window planes
    of 32 bases per word."""
    L = rd.shape[0]
    w2 = np.zeros(16, np.uint32)
    for i in range(L):
        w2[i // 16] |= np.uint32(int(rd[i]) << (2 * (i % 16)))
    nwin = win.shape[0]
    lo = np.zeros(16, np.uint32)
    hi = np.zeros(16, np.uint32)
    for b in range(min(nwin, 16 * 32)):
        lo[b // 32] |= np.uint32((int(win[b]) & 1) << (b % 32))
        hi[b // 32] |= np.uint32((int(win[b]) >> 1) << (b % 32))
    loc = C.c_int(0)
    err = po.lib().swo_banded_myers(w2.ctypes.data, L, e, lo.ctypes.data, hi.ctypes.data, rl, C.byref(loc))
    return err, loc.value


CONFIGS = [(150, 7, 164), (100, 5, 110), (250, 13, 276), (60, 3, 66), (200, 15, 230), (120, 0, 120),
           (150, 7, 157)]


@pytest.mark.parametrize("L,e,rl", CONFIGS)
def test_recurrence_equals_oracle(L, e, rl):
    rng = np.random.default_rng(L * 131 + e)
    win, rd = _cases(rng, 300, L, e, rl)
    error, loc, _, _ = _myers(win, rd, e, rl)
    for c in range(win.shape[0]):
        assert _oracle_myers(win[c], rd[c], e, rl) == (int(error[c]), int(loc[c])), c


@pytest.mark.parametrize("L,e,rl", CONFIGS)
def test_scan_minimum_never_drops_below(L, e, rl):
    rng = np.random.default_rng(L * 7 + e * 1009 + rl)
    win, rd = _cases(rng, 3000, L, e, rl)
    error, _, worst, mins = _myers(win, rd, e, rl)
    # no step's scan-range minimum is above the smallest final-scan cell
    assert int(worst.max()) <= 0
    # so the head's stop rule never drops a candidate that passes
    if L > 64:
        stopped = mins[63] > e
        assert not np.any(stopped & (error <= e))
        if 3 <= e <= 7:
            # and at the benchmark thresholds it stops a large share of the
            # failing ones (the point of the rule)
            assert stopped.sum() > 0.4 * (error > e).sum()
