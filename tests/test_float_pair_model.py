"""The float-pair arithmetic of the mixed form's solves (the operations of
csrc/float_pair.cuh) restated with numpy float32 on the CPU, to check the
precision the solves rely on: a pair holds about 48 significant bits, and
its sums, products, multiply-adds and quotients keep a relative error of a
few units of 2^-48.  The device code is checked against the oracle and the
FP64 solves by the GPU tests; this pins the formulas themselves."""
import numpy as np

f32 = np.float32
EPS48 = 2.0 ** -48


def fma32(a, b, c):
    # a*b is exact in float64 for float32 operands; one rounding to float32
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def quick(s, e):
    h = f32(s + e)
    return h, f32(e - f32(h - s))


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def add(a, b):
    s, e = two_sum(a[0], b[0])
    return quick(s, f32(e + f32(a[1] + b[1])))


def mul(a, b):
    p = f32(a[0] * b[0])
    e = fma32(a[0], b[0], -p)
    e = fma32(a[0], b[1], e)
    e = fma32(a[1], b[0], e)
    return quick(p, e)


def madd(a, b, c):
    p = f32(a[0] * b[0])
    e = fma32(a[0], b[0], -p)
    e = fma32(a[0], b[1], e)
    e = fma32(a[1], b[0], e)
    s, t = two_sum(c[0], p)
    return quick(s, f32(t + f32(e + c[1])))


def div(a, b):
    q1 = f32(a[0] / b[0])
    r = madd((f32(-q1), f32(0.0)), b, a)
    q2 = f32(r[0] / b[0])
    return quick(q1, q2)


def split(v):
    # as the device does it: hi the leading 24 significant bits (truncated),
    # lo the next 29 rounded to a float, then renormalised
    b = np.array([v], dtype=np.float64).view(np.uint64)[0]
    h64 = np.array([b & ~np.uint64((1 << 29) - 1)], dtype=np.uint64).view(np.float64)[0]
    return quick(f32(h64), f32(v - h64))


def val(p):
    return np.float64(p[0]) + np.float64(p[1])


def test_pair_operations_keep_48_bits():
    rng = np.random.default_rng(11)
    worst = {"split": 0.0, "add": 0.0, "mul": 0.0, "madd": 0.0, "div": 0.0}
    for _ in range(4000):
        x, y, z = rng.uniform(0.5, 2.0, 3) * 10.0 ** rng.integers(-12, 12, 3)
        x, y, z = x * rng.choice([-1, 1]), y * rng.choice([-1, 1]), z
        px, py, pz = split(x), split(y), split(z)
        worst["split"] = max(worst["split"], abs(val(px) - x) / abs(x))
        # references from the pairs' own values, so only the operation's
        # error is measured
        X, Y, Z = val(px), val(py), val(pz)
        s = X + Y
        if abs(s) > 1e-3 * max(abs(X), abs(Y)):        # away from cancellation
            worst["add"] = max(worst["add"], abs(val(add(px, py)) - s) / abs(s))
        worst["mul"] = max(worst["mul"], abs(val(mul(px, py)) - X * Y) / abs(X * Y))
        m = X * Y + Z
        if abs(m) > 1e-3 * abs(Z):
            worst["madd"] = max(worst["madd"], abs(val(madd(px, py, pz)) - m) / abs(m))
        worst["div"] = max(worst["div"], abs(val(div(px, py)) - X / Y) / abs(X / Y))
    assert worst["split"] <= EPS48
    for k in ("add", "mul", "madd", "div"):
        assert worst[k] <= 64 * EPS48, (k, worst[k])


def test_add_error_is_bounded_by_the_operands():
    """Under cancellation the sloppy sum's error stays within a few units of
    2^-48 of the larger operand, as the residual updates r - alpha A p need."""
    rng = np.random.default_rng(3)
    for _ in range(2000):
        x = rng.uniform(0.5, 2.0) * 10.0 ** rng.integers(-8, 8)
        y = -x * (1.0 + rng.uniform(-1e-6, 1e-6))
        px, py = split(x), split(y)
        X, Y = val(px), val(py)
        assert abs(val(add(px, py)) - (X + Y)) <= 8 * EPS48 * max(abs(X), abs(Y))
