"""The persistent ICP's exact merge with count bytes (acc_add with kAccCount, icp_await_totals in
supereight2_gb300/csrc/track.cu), restated in Python integers: every CTA splits its compensated
partial (hi, lo) of a term into a fixed-point integer part (2^-10) and fraction (2^-50) and adds
each, plus 2^56, into the 64-bit words of its copy (cta % 4); the words are never cleared, a
reader keeps the words as it last read them and takes the advances modulo 2^64. Checked here
over many iterations on three rotating buffers with partials up to the 2^38 limit, in random
arrival orders:
  - once every word's count byte has advanced by its copy's number of CTAs, the totals (the
    advances less their counts) equal the exact sum of the CTAs' fixed-point values;
  - no state with a CTA's addition still missing reads as complete;
  - partials of 2^38 or more are refused (the overflow flag), which keeps every copy's value
    below 2^55 in magnitude, under the count byte."""
from fractions import Fraction

import numpy as np

M64 = (1 << 64) - 1
COUNT = 1 << 56
COPIES = 4


def _fixed_split(v):
    """fixed_split (track.cu): |v| < 2^38 as I 2^-10 + F 2^-50 truncated toward zero, F in
    [0, 2^40); None outside the range."""
    b = int(np.array(v, np.float32).view(np.uint32))
    e = (b >> 23) & 0xff
    m = (b & 0x7fffff) | (0x800000 if e else 0)
    ee = e if e else 1
    if e == 0xff or ee > 164:
        return None
    i, f = 0, 0
    if ee >= 140:
        i = m << (ee - 140)
    elif ee >= 100:
        x = m << (ee - 100)
        i, f = x >> 40, x & ((1 << 40) - 1)
    elif 100 - ee < 24:
        f = m >> (100 - ee)
    if b >> 31:
        i, f = (-i - 1, (1 << 40) - f) if f else (-i, 0)
    return i, f


def _add(words, copy, hi, lo):
    """acc_add with the count: the two words of one term in one copy."""
    s_hi, s_lo = _fixed_split(hi), _fixed_split(lo)
    words[copy][0] = (words[copy][0] + s_hi[0] + s_lo[0] + COUNT) & M64
    words[copy][1] = (words[copy][1] + s_hi[1] + s_lo[1] + COUNT) & M64


def _read(words, prev, ngrid):
    """icp_await_totals for one term: (complete, A, B)."""
    ok, A, B = True, 0, 0
    for c in range(COPIES):
        n = ((ngrid - c + COPIES - 1) // COPIES) & 0xff
        dI = (words[c][0] - prev[c][0]) & M64
        dF = (words[c][1] - prev[c][1]) & M64
        cI, cF = ((dI + (COUNT >> 1)) & M64) >> 56, ((dF + (COUNT >> 1)) & M64) >> 56
        ok = ok and cI == n and cF == n
        vI = (dI - (cI << 56)) & M64
        A += vI - (1 << 64) if vI >> 63 else vI
        B += (dF - (cF << 56)) & M64
    return ok, A, B


def test_count_byte_merge_is_exact_and_detects_completion():
    rng = np.random.default_rng(21)
    ngrid = 152
    buffers = [[[0, 0] for _ in range(COPIES)] for _ in range(3)]
    prevs = [[[0, 0] for _ in range(COPIES)] for _ in range(3)]
    for phase in range(40):
        b = phase % 3
        words, prev = buffers[b], prevs[b]
        # partials of very different magnitudes, some at the edge of the range, some zero
        mag = 10.0 ** rng.integers(-12, 11, ngrid)
        his = (rng.standard_normal(ngrid) * mag).astype(np.float32)
        his[rng.integers(0, ngrid, 4)] = np.float32(2.7e11) * rng.choice([-1, 1], 4).astype(np.float32)
        his[rng.integers(0, ngrid, 4)] = 0.0
        los = (his * np.float32(2.0 ** -25) * rng.standard_normal(ngrid).astype(np.float32)).astype(np.float32)
        want = sum((Fraction(*map(int, (s[0], 1 << 10))) + Fraction(s[1], 1 << 50)
                    for h, l in zip(his, los) for s in (_fixed_split(h), _fixed_split(l))), Fraction(0))
        order = rng.permutation(ngrid)
        for k, cta in enumerate(order):
            _add(words, cta % COPIES, his[cta], los[cta])
            complete, A, B = _read(words, prev, ngrid)
            assert complete == (k == ngrid - 1), (phase, k)
        assert Fraction(A, 1 << 10) + Fraction(B, 1 << 50) == want
        prevs[b] = [list(w) for w in words]


def test_partials_past_the_range_are_refused():
    assert _fixed_split(np.float32(2.7e11)) is not None
    assert _fixed_split(np.float32(-2.8e11)) is None
    assert _fixed_split(np.float32(np.nan)) is None
    # the largest accepted partial keeps a copy of 128 CTAs below 2^55
    i, f = _fixed_split(np.nextafter(np.float32(2.0 ** 38), np.float32(0)))
    assert 128 * (abs(i) + 2) < 2 ** 55
