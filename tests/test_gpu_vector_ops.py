"""Vector updates and element-wise operations on the GPU (av / avbv / avbv_v,
element_op, vector_assign, vector_swap of linalg/vector_operations.hpp) against
numpy: bit-identical for the separately rounded products, quotients and sums
(numpy evaluates (x*a) + (z*b) with one rounding per operation, as the
reference's host loops do); pow and the unary functions within a few units in
the last place of numpy's (both sides call a math library)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V():
    import torch
    import vclgb
    torch.cuda.set_device(0)
    return vclgb


def _t(a):
    import torch
    return torch.tensor(a, device="cuda")


@pytest.mark.parametrize("dt", [np.float64, np.float32])
@pytest.mark.parametrize("ra,fa,rb,fb,acc,hasz", [
    (False, False, False, False, False, False),   # av
    (True, True, False, False, False, False),      # av, 1/(-alpha)
    (False, False, False, False, False, True),     # avbv
    (True, False, False, True, False, True),
    (False, True, True, False, True, True),        # avbv_v
    (True, True, True, True, True, True),
    (False, False, False, False, True, False)])    # y += x*alpha
def test_avbv_bit_exact(V, dt, ra, fa, rb, fb, acc, hasz):
    rng = np.random.default_rng(31)
    n = 100003
    x, z, y0 = (rng.uniform(-3, 3, n).astype(dt) for _ in range(3))
    a, b = dt(1.7320508), dt(-0.3141592)
    y = _t(y0.copy())
    V.avbv(y, _t(x), float(a), _t(z) if hasz else None, float(b), accumulate=acc,
           reciprocal_alpha=ra, flip_sign_alpha=fa, reciprocal_beta=rb, flip_sign_beta=fb)
    aa, bb = (-a if fa else a), (-b if fb else b)
    t = (x / aa) if ra else (x * aa)
    if hasz:
        t = t + ((z / bb) if rb else (z * bb))
    if acc:
        t = y0 + t
    assert np.array_equal(y.cpu().numpy(), t)


def test_avbv_strided_and_device_scalar(V):
    import torch
    rng = np.random.default_rng(32)
    n = 5000
    x = rng.uniform(-1, 1, 3 * n + 7)
    z = rng.uniform(-1, 1, 2 * n + 3)
    y0 = rng.uniform(-1, 1, 4 * n + 9)
    y = _t(y0.copy())
    alpha = torch.tensor(0.625, dtype=torch.float64, device="cuda")  # viennacl::scalar
    V.avbv((y, 9, 4), (_t(x), 7, 3), alpha, (_t(z), 3, 2), 2.5, n=n, accumulate=True)
    expect = y0.copy()
    expect[9::4][:n] = y0[9::4][:n] + (x[7::3][:n] * 0.625 + z[3::2][:n] * 2.5)
    assert np.array_equal(y.cpu().numpy(), expect)


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_element_binary(V, dt):
    rng = np.random.default_rng(33)
    n = 70001
    x = rng.uniform(0.1, 3, n).astype(dt)
    z = rng.uniform(-2, 2, n).astype(dt)
    assert np.array_equal(V.element_prod(_t(x), _t(z)).cpu().numpy(), x * z)
    assert np.array_equal(V.element_div(_t(x), _t(z)).cpu().numpy(), x / z)
    assert np.array_equal(V.element_div(_t(x), 3.0).cpu().numpy(), x / dt(3.0))
    assert np.array_equal(V.element_prod(2.5, _t(z)).cpu().numpy(), dt(2.5) * z)
    rtol = 4e-16 if dt == np.float64 else 4e-7
    np.testing.assert_allclose(V.element_pow(_t(x), _t(z)).cpu().numpy(), np.power(x, z), rtol=rtol)


DOMAINS = {"acos": (-0.99, 0.99), "asin": (-0.99, 0.99), "atanh": (-0.99, 0.99),
           "acosh": (1.0, 8.0), "log": (0.01, 50.0), "log2": (0.01, 50.0),
           "log10": (0.01, 50.0), "sqrt": (0.0, 50.0), "rsqrt": (0.01, 50.0)}


@pytest.mark.parametrize("name", ["abs", "acos", "acosh", "asin", "asinh", "atan", "atanh", "ceil",
                                  "cos", "cosh", "erf", "erfc", "exp", "exp2", "exp10", "fabs",
                                  "floor", "log", "log2", "log10", "round", "sin", "sinh", "sqrt",
                                  "tan", "tanh", "trunc", "rsqrt", "sign"])
def test_element_unary(V, name):
    rng = np.random.default_rng(34)
    lo, hi = DOMAINS.get(name, (-4.0, 4.0))
    x = rng.uniform(lo, hi, 40001)
    x[:4] = [lo, hi, 0.5 * (lo + hi), 2.5 if hi > 2.5 else hi]  # a half-way value for round
    ref = {"abs": np.abs, "fabs": np.fabs, "ceil": np.ceil, "floor": np.floor,
           "trunc": np.trunc, "sign": np.sign, "exp10": lambda v: np.exp(v * 2.302585092994045684),
           "rsqrt": lambda v: np.power(v, -0.5),
           "round": lambda v: np.where(v >= 0, np.floor(v + 0.5), np.ceil(v - 0.5)),
           "erf": lambda v: np.vectorize(__import__("math").erf)(v),
           "erfc": lambda v: np.vectorize(__import__("math").erfc)(v)}.get(name, getattr(np, name, None))
    if ref is None:
        ref = getattr(np, {"acosh": "arccosh", "asinh": "arcsinh", "atanh": "arctanh",
                           "acos": "arccos", "asin": "arcsin", "atan": "arctan"}[name])
    y = V.element_unary(name, _t(x)).cpu().numpy()
    exact = name in ("abs", "fabs", "ceil", "floor", "trunc", "sign", "round")
    if exact:
        assert np.array_equal(y, ref(x))
    else:
        np.testing.assert_allclose(y, ref(x), rtol=3e-15, atol=1e-300)


def test_assign_and_swap(V):
    rng = np.random.default_rng(35)
    a0, b0 = rng.uniform(-1, 1, 1000), rng.uniform(-1, 1, 1000)
    a, b = _t(a0.copy()), _t(b0.copy())
    V.vector_swap(a, b)
    assert np.array_equal(a.cpu().numpy(), b0) and np.array_equal(b.cpu().numpy(), a0)
    V.vector_assign((a, 1, 2), 4.25, n=400)
    e = b0.copy()
    e[1::2][:400] = 4.25
    assert np.array_equal(a.cpu().numpy(), e)
