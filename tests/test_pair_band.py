"""The mixed viscosity sweep decides "inside the radius" from FP32
coordinate pairs when their squared distance lies outside a band of 2^-16
(relative) around the exact FP64 threshold, and by the exact test inside it
(mps_gb300/csrc/sweeps.cu, k_explicit; the band is set up in capi.cu).  This
restates that decision on the host with numpy's IEEE FP32/FP64 arithmetic
and checks it against the exact test, sqrt_rn(dx^2 + dy^2) < re in FP64, on
seeded pairs of the 1M-particle dam break's coordinate range, concentrated
around the radius, so that the neighbour sets stay the exact ones."""
import math

import numpy as np


def _sq_threshold(re):
    # the smallest double t with sqrt_rn(t) >= re, as capi.cu computes it
    t = re * re
    while t > 0.0 and math.sqrt(t) >= re:
        t = np.nextafter(t, 0.0)
    while math.sqrt(t) < re:
        t = np.nextafter(t, np.inf)
    return float(t)


def test_pair_decision_matches_the_exact_test():
    rng = np.random.default_rng(20261204)
    l0 = 0.5 / 707
    re = 3.1 * l0
    t = _sq_threshold(re)
    f32 = np.float32
    fv_in = np.nextafter(f32(t * (1.0 - 2.0 ** -16)), f32(0.0))
    fv_out = np.nextafter(f32(t * (1.0 + 2.0 ** -16)), f32(np.inf))
    n = 400_000
    xi = rng.uniform(-0.004, 2.004, n)
    yi = rng.uniform(-0.004, 1.204, n)
    ang = rng.uniform(0.0, 2.0 * math.pi, n)
    # distances concentrated within 1e-6 relative of the radius, plus a spread
    near = rng.random(n) < 0.5
    rad = re * np.where(near, 1.0 + rng.normal(0.0, 1e-6, n), rng.uniform(0.3, 1.5, n))
    xj = xi + rad * np.cos(ang)
    yj = yi + rad * np.sin(ang)
    # exact decision (the reference's: FP64 differences, squares and sum, in that order)
    dx, dy = xj - xi, yj - yi
    d2 = dx * dx + dy * dy
    exact = d2 < t
    # FP32 pairs as the rebuild gather writes them: hi = f32(x), lo = f32(x - hi)
    def pair(v):
        hi = v.astype(f32)
        return hi, (v - hi.astype(np.float64)).astype(f32)
    hxi, lxi = pair(xi)
    hyi, lyi = pair(yi)
    hxj, lxj = pair(xj)
    hyj, lyj = pair(yj)
    fdx = (hxj - hxi) + (lxj - lxi)
    fdy = (hyj - hyi) + (lyj - lyi)
    d2f = fdx * fdx + fdy * fdy
    assert d2f.dtype == f32
    inside_f = d2f < fv_in
    outside_f = d2f > fv_out
    band = ~inside_f & ~outside_f
    decided = np.where(band, exact, inside_f)
    assert np.array_equal(decided, exact)
    # the band is narrow: for distances spread over the sweep's range the
    # exact FP64 test runs for a tiny share of the candidates only
    assert band[~near].mean() < 1e-3, band[~near].mean()
    # and the pairs' squared distance is within 2^-20 of the exact one
    rel = np.abs(d2f.astype(np.float64) - d2) / d2
    assert rel.max() < 2.0 ** -20, rel.max()
