"""Error bounds of the projection's first-try polynomial (csrc/fastpoly.cuh).

The projection accepts a polynomial angle only when a 1.2e-6 relative margin
around it stays inside one pixel, so its pixels equal those of the correctly
rounded angle as long as the polynomial is within that margin of the
correctly rounded float.  These tests evaluate the header's coefficients in
emulated FP32 (products and fma in extended precision, one rounding to
float) and check the bounds the header states, with the quotient of atan2
perturbed by the 2-ulp bound of the approximate division.
"""
import os
import re

import numpy as np

HDR = os.path.join(os.path.dirname(__file__), "..", "sloam_gb300", "csrc", "fastpoly.cuh")
MARGIN = 1.2e-6
f32 = np.float32


def _coeffs(name):
    src = open(HDR).read()
    m = re.search(r"#define %s((?:[^\n]*\\\n)*[^\n]*)" % name, src)
    assert m, name
    body = m.group(1).replace("\\\n", " ")
    return [f32(float(t.rstrip("f"))) for t in re.findall(r"[-+]?\d\.\d+e[-+]\d+f", body)]


def _fma(a, b, c):
    r = np.longdouble(a) * np.longdouble(b) + np.longdouble(c)
    return r.astype(f32)


def _horner(c, s):
    p = np.full_like(s, c[-1])
    for k in c[-2::-1]:
        p = _fma(p, s, k)
    return p


def _odd(c, a):
    return (a * _horner(c, (a * a).astype(f32))).astype(f32)


def _atan2(c, y, x, dq):
    ax, ay = np.abs(x), np.abs(y)
    a = (np.minimum(ax, ay) / np.maximum(ax, ay)).astype(f32)
    a = (a.astype(np.float64) * (1.0 + dq * 2.0 ** -23)).astype(f32)
    t = _odd(c, a)
    t = np.where(ay > ax, (f32(1.57079637) - t).astype(f32), t)
    t = np.where(x < 0, (f32(3.14159274) - t).astype(f32), t)
    return np.copysign(t, y).astype(f32)


def test_coefficients_parse():
    assert len(_coeffs("SG_ATAN_P")) == 9


def test_atan_polynomial_within_two_ulp():
    rng = np.random.default_rng(0)
    a = np.concatenate([f32(2.0) ** rng.uniform(-40, 0, 1_000_000).astype(f32),
                        rng.uniform(0, 1, 1_000_000).astype(f32), f32([1.0])]).astype(f32)
    a = a[a > 0]
    t = _odd(_coeffs("SG_ATAN_P"), a)
    ex = np.arctan(a.astype(np.float64))
    assert (np.abs(t - ex) / np.abs(ex)).max() < 1.5e-7


def test_yaw_within_margin_of_correctly_rounded():
    rng = np.random.default_rng(1)
    n = 1_000_000
    x = (rng.standard_normal(n) * 10 ** rng.uniform(-3, 2, n)).astype(f32)
    y = (rng.standard_normal(n) * 10 ** rng.uniform(-3, 2, n)).astype(f32)
    # axes, diagonals and octant edges
    x = np.concatenate([x, f32([1, -1, 1, -1, 3, -3, 1e-18, 1e18])])
    y = np.concatenate([y, f32([1, 1, -1, -1, 3 + 3e-7, -3, 1e18, 1e-18])])
    cr = np.arctan2(y.astype(np.float64), x.astype(np.float64)).astype(f32).astype(np.float64)
    c = _coeffs("SG_ATAN_P")
    worst = 0.0
    for dq in (-2.0, 0.0, 2.0):
        t = _atan2(c, y, x, dq).astype(np.float64)
        worst = max(worst, (np.abs(t - cr) / np.abs(t)).max())
    assert worst < 0.5 * MARGIN, worst
