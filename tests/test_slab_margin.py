"""The traversal's box culling must never reject a box the exact ray interval enters (results do not depend on
the tree only while culling is conservative). lighthouse2_gb300/csrc/traverse.cuh (Traversal::visit_node) computes
a slab distance from a plane byte q as t = v (2^15 a) + (b - 2^15 a - m) with v = 1 + q 2^-15, a = 2^e / d,
b = (p0 - O) / d, 1/d from the hardware reciprocal (at most 1 ulp off), and the per-axis margin
m = (2^-16 + 2^-19)(|b| + 255 |a|) + 2^-7 |a|. This test replays that float32 arithmetic (FMA as one rounding of the
exact product plus the addend) on random nodes and rays, near-parallel ones included, and checks against exact
rational distances that the widened entry distance stays at or below t - 2^-16 |t| and the exit distance at or
above t + 2^-16 |t|, the relative margin the triangle test relies on. A margin without the 2^-7 |a| term must fail
(the check has teeth)."""
from fractions import Fraction as Fr

import numpy as np

f32 = np.float32
SLAB = f32(2.0 ** -16 + 2.0 ** -19)


def fma(a, b, c):
    # product of two float32 is exact in float64 (48 bits); the sum is rounded to float64 and then to float32
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def widened(s, p0, O, invD, q, with_a_term=True):
    a = f32(s * invD)
    b = f32(f32(p0 - O) * invD)
    A = f32(a * f32(32768))
    base = f32(fma(f32(255), f32(abs(a)), f32(abs(b))) * SLAB)
    m = fma(f32(abs(a)), f32(0.0078125), base) if with_a_term else base
    c0 = f32(b - A)
    lo, hi = f32(c0 - m), f32(c0 + m)
    if not np.isfinite([a, b, A, m, lo, hi]).all():
        return None
    v = f32(1 + q * 2.0 ** -15)
    return fma(v, A, lo), fma(v, A, hi)


def cases(rng, n):
    for _ in range(n):
        s = f32(2.0 ** int(rng.integers(-12, 8)))
        p0, O = f32(rng.uniform(-1000, 1000)), f32(rng.uniform(-1000, 1000))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            d = f32(rng.uniform(-1, 1))
        elif kind == 1:   # almost parallel to the plane, down to the 1e-30 clamp
            d = f32(rng.choice([-1, 1]) * 10.0 ** rng.uniform(-30, -2))
        else:
            d = f32(rng.choice([-1, 1]) * 10.0 ** rng.uniform(-8, 0))
        if abs(d) < 1e-30 or d == 0:
            continue
        invD = f32(1) / d
        step = int(rng.integers(-1, 2))   # the hardware reciprocal: up to 1 ulp either way
        if step:
            invD = np.nextafter(invD, f32(np.inf) if step > 0 else f32(-np.inf))
        yield s, p0, O, d, invD, int(rng.integers(0, 256))


def check(n, seed, with_a_term):
    rng = np.random.default_rng(seed)
    bad = 0
    for s, p0, O, d, invD, q in cases(rng, n):
        r = widened(s, p0, O, invD, q, with_a_term)
        if r is None:
            continue
        tn, tf = r
        exact = (Fr(float(p0)) + q * Fr(float(s)) - Fr(float(O))) / Fr(float(d))
        if not (Fr(float(tn)) <= exact - abs(exact) / 65536 and Fr(float(tf)) >= exact + abs(exact) / 65536):
            bad += 1
    return bad


def test_slab_margin_is_conservative():
    assert check(20000, 7, True) == 0


def test_slab_margin_without_the_a_term_fails():
    assert check(3000, 7, False) > 0
