"""CSR triangular solves on the GPU (linalg::inplace_solve for the four tags, on
A and trans(A)) against the reference host backend's outputs and the oracle:
relative 2-norm error at most 1e-13 (the device substitutes level by level with
the entries pre-divided by their row's diagonal, so the rounding differs from
the reference's row-sequential loop)."""
import numpy as np
import pytest

import oracle
import vclgb_gen as gen
from conftest import rel_err

pytestmark = pytest.mark.gpu

TAGS = ["lower", "upper", "unit_lower", "unit_upper"]


@pytest.fixture(scope="module")
def V():
    import torch
    import vclgb
    torch.cuda.set_device(0)
    return vclgb


def _tag(V, name):
    return {"lower": V.lower_tag, "upper": V.upper_tag, "unit_lower": V.unit_lower_tag,
            "unit_upper": V.unit_upper_tag}[name]()


def _solve(V, A, b, tag, trans):
    import torch
    z = torch.tensor(b, dtype=torch.float64, device="cuda")
    V.inplace_solve(V.trans(A) if trans else A, z, _tag(V, tag))
    return z.cpu().numpy()


@pytest.mark.parametrize("trans", [0, 1])
@pytest.mark.parametrize("tag", TAGS)
@pytest.mark.parametrize("name", ["literal5", "convdiff_scaled", "lognormal"])
def test_inplace_solve_golden(V, golden, name, tag, trans):
    d = golden("trisolve.npz")
    rp, ci, v, b = d[name + "_rp"], d[name + "_ci"], d[name + "_v"], d[name + "_b"]
    A = V.compressed_matrix(rp, ci, v)
    z = _solve(V, A, b, tag, trans)
    assert rel_err(z, d["%s_tri_%s_%d" % (name, tag, trans)]) < 1e-13


@pytest.mark.parametrize("trans", [0, 1])
@pytest.mark.parametrize("tag", TAGS)
def test_inplace_solve_large_against_oracle(V, tag, trans):
    # a 2D grid (511 levels per triangle: runs of small levels in one block) and
    # a random matrix of 100k rows whose triangles have a few wide levels
    for rp, ci, v in (gen.convdiff2d(256, 256, peclet=5.0, shift=0.1),
                      gen.lognormal_random(100000, mu=1.5, sigma=0.8, hi=200, seed=23)):
        d = oracle.diag(rp, ci, v)
        rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp.astype(np.int64)))
        v = v / d[rows]  # unit diagonal: the unit solves stay bounded
        b = 1.0 + np.random.default_rng(24).uniform(0, 1, len(rp) - 1)
        A = V.compressed_matrix(rp, ci, v)
        z = _solve(V, A, b, tag, trans)
        assert rel_err(z, oracle.inplace_solve(rp, ci, v, b, tag, trans)) < 1e-12


def test_inplace_solve_values_refreshed_and_repeatable(V):
    # the level structure is cached per matrix; the values are read at every call
    import torch
    rp, ci, v = gen.convdiff2d(40, 40, peclet=10.0, shift=0.05)
    vals = torch.tensor(v, device="cuda")
    rpd = torch.tensor(rp.astype(np.int32), device="cuda")
    cid = torch.tensor(ci.astype(np.int32), device="cuda")
    A = V.compressed_matrix(rpd, cid, vals)
    assert A.values.data_ptr() == vals.data_ptr()  # wrapped, not copied
    b = 1.0 + np.random.default_rng(25).uniform(0, 1, len(rp) - 1)
    z1 = _solve(V, A, b, "lower", 0)
    assert np.array_equal(z1, _solve(V, A, b, "lower", 0))
    vals.mul_(2.0)
    z2 = _solve(V, A, b, "lower", 0)
    assert rel_err(z2, oracle.inplace_solve(rp, ci, 2.0 * v, b, "lower", 0)) < 1e-13


def test_inplace_solve_rejects_bad_arguments(V):
    import torch
    rp, ci, v = gen.laplace2d(8, 8)
    A = V.compressed_matrix(rp, ci, v)
    z = torch.ones(len(rp) - 1, dtype=torch.float64, device="cuda")
    with pytest.raises(V.VclgbError):
        V.inplace_solve(A, z, 7)
    with pytest.raises(V.VclgbError):
        V.inplace_solve(A, z.float(), V.lower_tag())
