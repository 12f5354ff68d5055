"""Accuracy of the project's fixed-order fp32 transcendentals (csrc/gi_math.h)
against the C library in double precision (no GPU).  The CUDA kernels and the
fp32 oracle evaluate exactly these functions."""
import numpy as np
import pytest


def _ulp_err(got, ref):
    got = got.astype(np.float64)
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    return np.abs(got - ref) / ulp


@pytest.mark.parametrize("fn,lo,hi,ref,max_ulp", [
    ("log", 1e-30, 1e30, np.log, 4), ("log2", 1e-30, 1e30, np.log2, 4),
    ("exp", -80, 80, np.exp, 4), ("exp2", -120, 120, np.exp2, 4),
    ("sin", -12, 12, np.sin, None), ("cos", -12, 12, np.cos, None),
])
def test_unary_accuracy(oracle, fn, lo, hi, ref, max_ulp):
    rng = np.random.default_rng(1)
    if fn in ("log", "log2"):
        x = np.exp(rng.uniform(np.log(lo), np.log(hi), 200000)).astype(np.float32)
    else:
        x = rng.uniform(lo, hi, 200000).astype(np.float32)
    got = oracle.math_batch(fn, x)
    r = ref(x.astype(np.float64))
    if max_ulp is None:  # sin/cos: absolute error near the zeros
        assert np.max(np.abs(got - r)) < 3e-7
    else:
        assert np.max(_ulp_err(got, r)) <= max_ulp


def test_atan2_accuracy_and_quadrants(oracle):
    rng = np.random.default_rng(2)
    y = rng.normal(size=200000).astype(np.float32) * np.float32(10) ** rng.integers(-3, 3, 200000)
    x = rng.normal(size=200000).astype(np.float32) * np.float32(10) ** rng.integers(-3, 3, 200000)
    got = oracle.math_batch("atan2", y.astype(np.float32), x.astype(np.float32))
    r = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.max(np.abs(got - r)) < 5e-7
    sp = np.array([[0.0, 1.0], [0.0, -1.0], [1.0, 0.0], [-1.0, 0.0], [np.inf, np.inf], [-np.inf, 1.0]], np.float32)
    g = oracle.math_batch("atan2", sp[:, 0], sp[:, 1])
    assert np.allclose(g, np.arctan2(sp[:, 0], sp[:, 1]), atol=1e-7)


def test_pow_accuracy(oracle):
    rng = np.random.default_rng(3)
    b = rng.uniform(0.0, 4.0, 100000).astype(np.float32)
    e = rng.uniform(0.0, 30.0, 100000).astype(np.float32)
    got = oracle.math_batch("pow", b, e)
    r = np.power(b.astype(np.float64), e.astype(np.float64))
    ok = r < 1e30
    assert np.max(np.abs(got[ok] - r[ok]) / np.maximum(r[ok], 1e-30)) < 2e-5
    assert oracle.math_batch("pow", np.float32([0.0, 1.0]), np.float32([2.2, 5.0])).tolist() == [0.0, 1.0]


def test_special_values(oracle):
    assert oracle.math_batch("log", np.float32([0.0]))[0] == -np.inf
    assert np.isnan(oracle.math_batch("log", np.float32([-1.0]))[0])
    assert oracle.math_batch("log", np.float32([1.0]))[0] == 0.0
    assert oracle.math_batch("exp", np.float32([-200.0]))[0] == 0.0
    assert oracle.math_batch("exp", np.float32([0.0]))[0] == 1.0
    assert oracle.math_batch("log2", np.float32([8.0]))[0] == 3.0
