"""ILU0 on the GPU: factors bit-identical to the reference's sequential host
factorisation, level sets identical to level_scheduling_setup_L/U, and the
level-scheduled apply within 1e-13 of the reference."""
import numpy as np
import pytest

import oracle
import vclgb_gen as gen
from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V():
    import torch
    import vclgb
    torch.cuda.set_device(0)
    return vclgb


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


def test_golden_factors_and_levels(V, golden):
    import torch
    d = golden("ilu0_convdiff.npz")
    rp, ci, v = d["rp"], d["ci"], d["v"]
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    P = V.ilu0_precond(A, True)
    inf = P.info()
    assert np.array_equal(P.export(0, len(v), torch.float64).cpu().numpy(), d["lu"])
    assert np.array_equal(P.export(1, n, torch.float64).cpu().numpy(), d["udiag"])
    for tri, base, levels, rows, nnz in (("L", 2, inf.num_levels_L, inf.rows_L, inf.nnz_L),
                                         ("U", 7, inf.num_levels_U, inf.rows_U, inf.nnz_U)):
        assert np.array_equal(_u32(P.export(base, levels + 1, torch.int32)), d[tri + "_level_ptr"])
        assert np.array_equal(_u32(P.export(base + 1, rows, torch.int32)), d[tri + "_row_index"])
        assert np.array_equal(_u32(P.export(base + 2, rows + 1, torch.int32)), d[tri + "_row_ptr"])
        assert np.array_equal(_u32(P.export(base + 3, nnz, torch.int32)), d[tri + "_cols"])
        assert np.array_equal(P.export(base + 4, nnz, torch.float64).cpu().numpy(),
                              d[tri + "_vals"])
    z = torch.tensor(d["b"], device="cuda")
    P.apply(z)
    assert rel_err(z.cpu().numpy(), d["z"]) < 1e-13


def _scrambled(rp, ci, v, seed):
    # P A P^T for a random P: each row's lower/upper entries then fall into
    # several levels, so a row is updated at more than one level
    sp = pytest.importorskip("scipy.sparse")
    n = len(rp) - 1
    perm = np.random.default_rng(seed).permutation(n)
    B = sp.csr_matrix((v, ci, rp), shape=(n, n))[perm][:, perm].tocsr()
    B.sort_indices()
    return B.indptr.astype(np.uint32), B.indices.astype(np.uint32), B.data.astype(np.float64)


def _random_dominant(n, per_row, seed):
    # random pattern with up to per_row off-diagonals a row plus a dominant
    # diagonal: rows with more entries in one level than the apply prefetches
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(seed)
    r = np.repeat(np.arange(n), per_row)
    c = rng.integers(0, n, n * per_row)
    M = sp.coo_matrix((rng.uniform(-1, 0, n * per_row), (r, c)), shape=(n, n)).tocsr()
    M = M + M.T
    M = M + sp.diags(np.asarray(abs(M).sum(axis=1)).ravel() + 1.0)
    M = M.tocsr()
    M.sum_duplicates()
    M.sort_indices()
    return M.indptr.astype(np.uint32), M.indices.astype(np.uint32), M.data.astype(np.float64)


@pytest.mark.parametrize("case", ["lap3d", "lap3d_40", "lap3d_96", "diffusion2d", "scrambled2d",
                                  "scrambled3d", "random"])
def test_factors_match_oracle(V, case):
    # lap3d (levels of at most 400 rows) runs one block; lap3d_40 (up to ~1,200
    # rows a level) a cluster of 128-thread CTAs, or one block and grid-wide
    # levels where clusters cannot be launched; lap3d_96 (up to ~6,900 rows) a
    # cluster of 512-thread CTAs; the scrambled and random patterns have rows
    # spread over several levels
    import torch
    if case == "lap3d":
        rp, ci, v = gen.laplace3d(20)
    elif case == "lap3d_40":
        rp, ci, v = gen.laplace3d(40)
    elif case == "lap3d_96":
        rp, ci, v = gen.laplace3d(96)
    elif case == "scrambled2d":
        rp, ci, v = _scrambled(*gen.convdiff2d(40, 40, peclet=10.0, shift=0.01), seed=5)
    elif case == "scrambled3d":
        rp, ci, v = _scrambled(*gen.laplace3d(16), seed=6)
    elif case == "random":
        rp, ci, v = _random_dominant(3000, 8, seed=7)
    else:
        rp, ci, v, _ = gen.diffusion2d_edges(60)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    P = V.ilu0_precond(A)
    lu = oracle.ilu0_factor(rp, ci, v)
    assert np.array_equal(P.export(0, len(v), torch.float64).cpu().numpy(), lu)
    b = gen.rhs_uniform(n, 1)
    z = torch.tensor(b, device="cuda")
    P.apply(z)
    assert rel_err(z.cpu().numpy(), oracle.ilu0_apply(rp, ci, v, b)) < 1e-13
