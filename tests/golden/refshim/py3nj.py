"""Wigner 3j symbols, exact: Racah's single-sum formula evaluated in rational
arithmetic, rounded to float once at the end. Arguments are doubled integers, as
in py3nj.wigner3j."""
from fractions import Fraction
from functools import lru_cache
from math import factorial, sqrt

import numpy as np


@lru_cache(maxsize=None)
def _three_j(tj1, tj2, tj3, tm1, tm2, tm3):
    if tm1 + tm2 + tm3 != 0:
        return 0.0
    if any(abs(m) > j for m, j in ((tm1, tj1), (tm2, tj2), (tm3, tj3))):
        return 0.0
    if any((j + m) % 2 for m, j in ((tm1, tj1), (tm2, tj2), (tm3, tj3))):
        return 0.0
    if tj3 > tj1 + tj2 or tj3 < abs(tj1 - tj2) or (tj1 + tj2 + tj3) % 2:
        return 0.0
    j1, j2, j3 = Fraction(tj1, 2), Fraction(tj2, 2), Fraction(tj3, 2)
    m1, m2, m3 = Fraction(tm1, 2), Fraction(tm2, 2), Fraction(tm3, 2)
    f = lambda x: factorial(int(x))
    tri = Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3), f(j1 + j2 + j3 + 1))
    pre = tri * f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3)
    tmin = int(max(0, j2 - j3 - m1, j1 - j3 + m2))
    tmax = int(min(j1 + j2 - j3, j1 - m1, j2 + m2))
    s = Fraction(0)
    for t in range(tmin, tmax + 1):
        den = (f(t) * f(j3 - j2 + t + m1) * f(j3 - j1 + t - m2) * f(j1 + j2 - j3 - t)
               * f(j1 - t - m1) * f(j2 - t + m2))
        s += Fraction((-1) ** t, den)
    if s == 0:
        return 0.0
    phase = -1 if int(j1 - j2 - m3) % 2 else 1
    sign = phase * (1 if s > 0 else -1)
    return sign * sqrt(float(pre * s * s))


def wigner3j(tj1, tj2, tj3, tm1, tm2, tm3, ignore_invalid=False):
    args = [np.atleast_1d(np.asarray(x)).astype(np.int64) for x in (tj1, tj2, tj3, tm1, tm2, tm3)]
    n = max(len(a) for a in args)
    args = [np.broadcast_to(a, (n,)) for a in args]
    return np.array([_three_j(*(int(a[i]) for a in args)) for i in range(n)], dtype=np.float64)
