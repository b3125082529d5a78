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


@pytest.mark.parametrize("case", ["lap3d", "diffusion2d"])
def test_factors_match_oracle(V, case):
    import torch
    if case == "lap3d":
        rp, ci, v = gen.laplace3d(20)
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
