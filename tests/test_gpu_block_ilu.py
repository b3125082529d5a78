"""block_ilu_precond<compressed_matrix, ilu0_tag> on the GPU: the blocks'
ILU0 factors bit-identical to the reference's, the apply within 1e-13 of the
oracle (which applies every entry of U; the reference's apply skips U's last
column, see the oracle's pin tests), BiCGStab preconditioned by it."""
import numpy as np
import pytest

import oracle
import vclgb_gen as gen
from conftest import iters_close, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V():
    import torch
    import vclgb
    torch.cuda.set_device(0)
    return vclgb


def _np(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("nb", [1, 8, 37])
def test_golden_factors_and_apply(V, golden, nb):
    import torch
    d = golden("block_ilu.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    P = V.block_ilu_precond(A, num_blocks=nb)
    lu = d["lu_%d" % nb]
    assert np.array_equal(_np(P.export(0, len(lu), torch.float64)), lu)
    B = oracle.block_ilu0(d["rp"], d["ci"], d["v"], num_blocks=nb)
    z = _np(P.apply(torch.tensor(d["b"], device="cuda")))
    assert rel_err(z, oracle.block_ilu0_apply(B, d["b"])) < 1e-13


@pytest.mark.parametrize("case", ["lap3d", "scrambled", "lognormal"])
@pytest.mark.parametrize("nb", [3, 64, 1000])
def test_matches_oracle(V, case, nb):
    import torch
    if case == "lap3d":
        rp, ci, v = gen.laplace3d(20)
    elif case == "scrambled":
        sp = pytest.importorskip("scipy.sparse")
        rp, ci, v = gen.convdiff2d(45, 40, peclet=10.0, shift=0.01)
        n = len(rp) - 1
        perm = np.random.default_rng(3).permutation(n)
        M = sp.csr_matrix((v, ci, rp), shape=(n, n))[perm][:, perm].tocsr()
        M.sort_indices()
        rp, ci, v = M.indptr.astype(np.uint32), M.indices.astype(np.uint32), M.data
    else:
        rp, ci, v = gen.lognormal_random(3000, mu=2.0, sigma=1.0, hi=200, seed=9)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    P = V.block_ilu_precond(A, num_blocks=nb)
    B = oracle.block_ilu0(rp, ci, v, num_blocks=nb)
    assert np.array_equal(_np(P.export(0, B["nnz"], torch.float64)), B["lu"][:B["nnz"]])
    b = gen.rhs_uniform(n, 5)
    z = _np(P.apply(torch.tensor(b, device="cuda")))
    assert rel_err(z, oracle.block_ilu0_apply(B, b)) < 1e-13


def test_custom_boundaries(V):
    # block_boundaries in any order, empty blocks allowed; gaps and overlaps rejected
    import torch
    rp, ci, v = gen.convdiff2d(30, 30, peclet=5.0, shift=0.02)
    n = len(rp) - 1
    bounds = [(500, 900), (0, 120), (120, 120), (120, 500)]
    A = V.compressed_matrix(rp, ci, v)
    P = V.block_ilu_precond(A, block_boundaries=bounds)
    B = oracle.block_ilu0(rp, ci, v, bounds=sorted(bounds))
    b = gen.rhs_uniform(n, 8)
    assert np.array_equal(_np(P.export(0, B["nnz"], torch.float64)), B["lu"][:B["nnz"]])
    assert rel_err(_np(P.apply(torch.tensor(b, device="cuda"))), oracle.block_ilu0_apply(B, b)) < 1e-13
    for bad in ([(0, 100), (150, 900)], [(0, 500), (400, 900)], [(0, 899)]):
        with pytest.raises(V.VclgbError) as e:
            V.block_ilu_precond(A, block_boundaries=bad)
        assert e.value.status == V.INVALID_ARGUMENT
    with pytest.raises(V.VclgbError) as e:
        V.block_ilu_precond(A, num_blocks=0)
    assert e.value.status == V.INVALID_ARGUMENT


def test_solve(V, golden):
    # BiCGStab + block ILU0 (8 blocks): iterations as the oracle's (which
    # applies U's last column), solution as the reference's
    d = golden("block_ilu.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    tag = V.bicgstab_tag(1e-10, 2000)
    x = _np(V.solve(A, d["b"], tag, V.block_ilu_precond(A, num_blocks=8)))
    _, it, _ = oracle.solve("bicgstab", d["rp"], d["ci"], d["v"], d["b"], 1e-10, 2000, "bilu8")
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), it)
    assert rel_err(x, d["x_bicgstab_bilu8"]) < 1e-6
