"""CPU restatements of two numerical devices of the GPU's Fisher tail sum
(gepicount_gb300/csrc/device.cuh), checked on random hypergeometric tables:

* the float-float tail walk (fisher_walk_ff, then fisher_walk_tail): terms and
  their sum as FP32 pairs hi + lo built from Dekker's exact product and
  Knuth's exact sum, FP32 alone once a term adds < 1e-9 of the sum -- against
  the exact rational sum of the same terms;
* the far-side search (fisher_lnp): two FP32 bisections on the float
  log-factorial table bracket the first term that passes R's rule, and an
  FP64 bisection decides it inside the bracket -- against the plain FP64
  bisection.

FP32 arithmetic is numpy float32 (IEEE round to nearest).  The fused
multiply-add is the exact product and sum, rounded to FP64 and then to FP32
(rarely a last-bit difference from one rounding).  The reciprocal is IEEE
division where the device takes the approximate one; the remainder
correction that follows absorbs either.  The GPU tests check the device
values themselves against the oracle (|d ln p| <= 1e-9); these check the
methods behind them over wider sizes (N up to 10^6)."""
import math
import random
from fractions import Fraction

import numpy as np

f32 = np.float32


def _fma(a, b, c):
    return f32(float(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))))


def _fast_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def _two_sum(a, b):
    s = f32(a + b)
    v = f32(s - a)
    return s, f32(f32(a - f32(s - v)) + f32(b - v))


def _add(a, b):
    s, e = _two_sum(a[0], b[0])
    return _fast_sum(s, f32(e + f32(a[1] + b[1])))


def _mul(a, b):
    p = f32(a[0] * b[0])
    e = _fma(a[0], b[0], -p)
    e = _fma(a[0], b[1], _fma(a[1], b[0], e))
    return _fast_sum(p, e)


def _two_prod(a, b):
    p = f32(a * b)
    return p, _fma(a, b, -p)


def _div(a, b):
    rb = f32(f32(1) / b[0])
    q1 = f32(a[0] * rb)
    p, pe = _two_prod(q1, b[0])
    r = f32(a[0] - p)
    r = f32(r + f32(a[1] - pe))
    r = _fma(-q1, b[1], r)
    return _fast_sum(q1, f32(r * rb))


def _split(x):
    h = f32(x)
    return h, f32(x - float(h))


def _walk_ff(x, step, x_end, ratio4):
    """fisher_walk_ff from S0 = t0 = 1 (the observed term), then the FP32 tail."""
    S, t, low = _split(1.0), _split(1.0), False
    while x != x_end:
        a, b, c, e = ratio4(x)
        x += step
        t = _mul(t, _div(_two_prod(f32(a), f32(b)), _two_prod(f32(c), f32(e))))
        S = _add(S, t)
        if t[0] < f32(1e-9) * S[0]:
            low = True
            break
    Sd = float(S[0]) + float(S[1])
    if not low:
        return Sd
    tt, St, stop = t[0], f32(0), f32(1e-17 * Sd)
    while x != x_end:
        a, b, c, e = ratio4(x)
        x += step
        tt = f32(tt * f32(f32(f32(a) * f32(b)) / f32(f32(c) * f32(e))))
        St = f32(St + tt)
        if tt < stop:
            break
    return Sd + float(St)


def _walk_exact(x, step, x_end, ratio4):
    S = t = Fraction(1)
    while x != x_end:
        a, b, c, e = ratio4(x)
        x += step
        t = t * a * b / (c * e)
        S += t
        if t < S * Fraction(1, 10**19):
            break
    return S


def _table(rng, sizes):
    while True:
        N = rng.choice(sizes)
        r1 = rng.randint(1, N - 1)
        c1 = rng.randint(1, N - 1)
        r2 = N - r1
        lo, hi = max(0, c1 - r2), min(c1, r1)
        if lo < hi:
            return N, r1, r2, c1, lo, hi


def test_float_float_tail_walk_matches_exact_sums():
    rng = random.Random(2)
    worst = 0.0
    for _ in range(150):
        N, r1, r2, c1, lo, hi = _table(rng, [200, 2000, 4000, 10000, 100000, 1000000])
        xm = min(max((r1 + 1) * (c1 + 1) // (N + 2), lo), hi)
        # half the observations within a few standard deviations of the mode,
        # where the walks are long
        sd = math.sqrt(max(1.0, r1 * c1 * (N - r1) * (N - c1) / (N * N * (N - 1.0))))
        xo = rng.randint(lo, hi) if rng.random() < 0.5 else \
            min(max(xm + int(rng.uniform(-6, 6) * sd), lo), hi)
        up = lambda x: (r1 - x, c1 - x, x + 1, r2 - c1 + x + 1)
        down = lambda x: (x, r2 - c1 + x, r1 - x + 1, c1 - x + 1)
        # the walk away from the mode, where terms fall
        step, x_end, ratio = (-1, lo, down) if xo <= xm else (1, hi, up)
        got = _walk_ff(xo, step, x_end, ratio)
        want = _walk_exact(xo, step, x_end, ratio)
        worst = max(worst, float(abs(Fraction(got) - want) / want))
    assert worst < 1e-11, worst  # the p-values are held to 1e-9


def test_fp32_bracketed_search_finds_the_fp64_bisection_term():
    rng = random.Random(5)
    nmax = 200001
    lf = np.array([math.lgamma(n + 1) for n in range(nmax)], dtype=np.float64)
    lf32 = lf.astype(np.float32)
    checked = 0
    while checked < 1500:
        N, r1, r2, c1, lo, hi = _table(rng, [50, 200, 2000, 4000, 10000, 100000, 200000])
        xm = min(max((r1 + 1) * (c1 + 1) // (N + 2), lo), hi)
        xo = rng.randint(lo, hi) if rng.random() < 0.5 else min(max(xm + rng.randint(-5, 5), lo), hi)
        K = lf[r1] + lf[r2] + lf[c1] + lf[N - c1] - lf[N]

        def lpx(x):
            return K - lf[x] - lf[r1 - x] - lf[c1 - x] - lf[r2 - c1 + x]

        lim = lpx(xo) + 9.99999950000003e-08
        E = f32(f32(2e-6) * lf32[N] + f32(1e-6))
        gc = f32(K - lim)

        def g32(x):
            return f32(f32(f32(f32(gc - lf32[x]) - lf32[r1 - x]) - lf32[c1 - x]) - lf32[r2 - c1 + x])

        if xo <= xm:
            a, b = xm + 1, hi
            if a > b or lpx(b) > lim:
                continue
            l, h = a, b
            while l < h:
                mid = (l + h) >> 1
                l, h = (l, mid) if lpx(mid) <= lim else (mid + 1, h)
            plain = l
            l, h = a, b
            while l < h:
                mid = (l + h) >> 1
                l, h = (l, mid) if g32(mid) <= E else (mid + 1, h)
            t0, h = l, b
            while l < h:
                mid = (l + h) >> 1
                l, h = (l, mid) if g32(mid) < -E else (mid + 1, h)
            l = t0
            while l < h:
                mid = (l + h) >> 1
                l, h = (l, mid) if lpx(mid) <= lim else (mid + 1, h)
        else:
            a, b = lo, xm - 1
            if a > b or lpx(a) > lim:
                continue
            l, h = a, b
            while l < h:
                mid = (l + h + 1) >> 1
                l, h = (mid, h) if lpx(mid) <= lim else (l, mid - 1)
            plain = l
            l, h = a, b
            while l < h:
                mid = (l + h + 1) >> 1
                l, h = (mid, h) if g32(mid) <= E else (l, mid - 1)
            t0, l = h, a
            while l < h:
                mid = (l + h + 1) >> 1
                l, h = (mid, h) if g32(mid) < -E else (l, mid - 1)
            h = t0
            while l < h:
                mid = (l + h + 1) >> 1
                l, h = (mid, h) if lpx(mid) <= lim else (l, mid - 1)
        assert l == plain, (N, r1, c1, xo)
        checked += 1
