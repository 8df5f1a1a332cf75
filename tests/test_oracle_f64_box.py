"""The double walks' FP32 query box holds the exact double query box (host check of the rule).

A double query (centre P, padded radius rs = rc + pad rounded up) looks for records inside the
FP32 box of each image t.  The kernels form that box from the query rounded to nearest (Pf) and
the image choice's radius rsf = ru(ru(rs) + 2 ulp(M)), every step rounded away from the centre:
lo = rd(rd(Pf + t) - rsf), hi = ru(ru(Pf + t) + rsf).  A record (the point rounded down to a
float) of any point within rs of P + t must lie inside it, so the box must hold the exact box
[P + t - rs, P + t + rs].  Checked here in exact rational arithmetic on adversarial inputs:
centres next to floats and to binade edges, the 27 image vectors of the benchmark's box, cutoffs
from 0.5 to 3.
"""
import fractions
import math

import numpy as np

F = fractions.Fraction


def _f32_down(x: F) -> float:
    """Largest float32 not above the rational x."""
    f = float(np.float32(float(x)))
    while F(f) > x:
        f = float(np.nextafter(np.float32(f), np.float32(-np.inf)))
    while F(float(np.nextafter(np.float32(f), np.float32(np.inf)))) <= x:
        f = float(np.nextafter(np.float32(f), np.float32(np.inf)))
    return f


def _f32_up(x: F) -> float:
    """Smallest float32 not below the rational x."""
    return -_f32_down(-x)


def _f32_nearest(x: float) -> float:
    return float(np.float32(x))


def _ulp_of(x: float) -> float:
    """The kernels' ulp_of: 2^e * 2^-23 for the binade of the float x."""
    m, e = math.frexp(x)       # x = m * 2^e, m in [0.5, 1)
    return math.ldexp(1.0, e - 1 - 23)


def _f64_up(x: F) -> float:
    """Smallest double not below the rational x."""
    d = float(x)
    if F(d) < x:
        d = math.nextafter(d, math.inf)
    return d


def _box(P, t, rs_d, M):
    """The kernels' FP32 box of image t (query_box_f32 with screen_f64's Pf and rsf)."""
    uM = _ulp_of(max(M, 1.17549435e-38))
    rsf = _f32_up(F(_f32_up(F(rs_d))) + F(2.0 * uM))
    lo, hi = [], []
    for k in range(3):
        pf = _f32_nearest(P[k])
        lo.append(_f32_down(F(_f32_down(F(pf) + F(t[k]))) - F(rsf)))
        hi.append(_f32_up(F(_f32_up(F(pf) + F(t[k]))) + F(rsf)))
    return lo, hi


def test_fp32_query_box_holds_the_exact_double_box():
    rng = np.random.default_rng(2024)
    L = float(np.float32(270.25))
    images = [(ix * L, iy * L, iz * L) for ix in (-1, 0, 1) for iy in (-1, 0, 1) for iz in (-1, 0, 1)]
    cases = 0
    for trial in range(400):
        rc = float(rng.uniform(0.5, 3.0))
        pad = 16.0 * math.ldexp(1.0, math.frexp(2 * L + rc)[1] - 24) + rc * 1e-6
        rs_d = _f64_up(F(rc) + F(pad))
        P = []
        for k in range(3):
            kind = trial % 4
            if kind == 0:      # next to a float
                f = float(np.float32(rng.uniform(0, L)))
                P.append(f + rng.choice([-1, 1]) * rng.uniform(0, 1) * math.ulp(f) * 2 ** 28)
            elif kind == 1:    # next to a binade edge
                e = 2.0 ** int(rng.integers(0, 9))
                P.append(min(max(e * (1 + rng.uniform(-1e-7, 1e-7)), 0.0), L))
            else:
                P.append(float(rng.uniform(0, L)))
        M = max(max(abs(_f32_nearest(p)) for p in P), L)
        for t in images:
            lo, hi = _box(P, t, rs_d, M)
            for k in range(3):
                c = F(P[k]) + F(t[k])
                assert F(lo[k]) <= c - F(rs_d), (P, t, k)
                assert F(hi[k]) >= c + F(rs_d), (P, t, k)
                # and it is no more than a few ulps wider than the exact box rounded outward
                assert F(hi[k]) - F(lo[k]) <= 2 * F(rs_d) + 16 * F(_ulp_of(max(M, 1.0)))
            cases += 1
    assert cases == 400 * 27
