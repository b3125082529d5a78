"""Chow-Patel ILU0 / IC0 on the GPU: the Neumann matrices and diagonals
bit-identical to the reference host backend's detail::precondition (the zero
diagonal entries the reference stores are left out on the device), the apply
within 1e-13 of the reference's, and BiCGStab / CG preconditioned by them
against the reference's runs."""
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


def _u32(t):
    return _np(t).view(np.uint32)


def _check_against(P, F):
    """Device Neumann matrices and diagonals against full-pattern host ones."""
    for base, tri in ((0, "l"), (4, "u")):
        rp, ci, v = oracle.strip_diagonal(F[tri + "_rp"], F[tri + "_ci"], F[tri + "_v"])
        assert np.array_equal(_u32(P.export(base)), rp)
        assert np.array_equal(_u32(P.export(base + 1)), ci)
        assert np.array_equal(_np(P.export(base + 2)), v)
        assert np.array_equal(_np(P.export(base + 3)), F["diag_" + tri])


@pytest.mark.parametrize("mat", ["cd", "sd"])
@pytest.mark.parametrize("sweeps,iters", [(3, 2), (1, 4)])
def test_golden(V, golden, mat, sweeps, iters):
    import torch
    d = golden("chow_patel.npz")
    rp, ci, v = (d["cp"], d["cc"], d["cv"]) if mat == "cd" else (d["sp"], d["sc"], d["sv"])
    t = "%s_%d_%d_" % (mat, sweeps, iters)
    A = V.compressed_matrix(rp, ci, v)
    tag = V.chow_patel_tag(sweeps, iters)
    for cls, pre, upre, z in ((V.chow_patel_ilu_precond, "cpl", "cpu", "cp_ilu_z"),
                              (V.chow_patel_icc_precond, "icl", "iclt", "cp_icc_z")):
        P = cls(A, tag)
        inf = P.info()
        assert (inf.sweeps, inf.jacobi_iters) == (sweeps, iters)
        F = {"l_rp": d[t + pre + "_rp"], "l_ci": d[t + pre + "_ci"], "l_v": d[t + pre + "_v"],
             "diag_l": d[t + pre + "_diag"], "u_rp": d[t + upre + "_rp"],
             "u_ci": d[t + upre + "_ci"], "u_v": d[t + upre + "_v"],
             "diag_u": d[t + ("cpu_diag" if pre == "cpl" else "icl_diag")]}
        _check_against(P, F)
        vec = torch.tensor(d["b_" + mat], device="cuda")
        assert rel_err(_np(P.apply(vec)), d[t + z]) < 1e-13


def _scrambled(rp, ci, v, seed):
    sp = pytest.importorskip("scipy.sparse")
    n = len(rp) - 1
    perm = np.random.default_rng(seed).permutation(n)
    B = sp.csr_matrix((v, ci, rp), shape=(n, n))[perm][:, perm].tocsr()
    B.sort_indices()
    return B.indptr.astype(np.uint32), B.indices.astype(np.uint32), B.data.astype(np.float64)


@pytest.mark.parametrize("case", ["lap3d", "diffusion2d", "convdiff_scrambled", "lognormal"])
@pytest.mark.parametrize("sweeps,iters", [(3, 2), (0, 1), (2, 0)])
def test_matches_oracle(V, case, sweeps, iters):
    # larger and irregular patterns (rows of up to a few hundred entries), no
    # sweep, no Jacobi step: factors bit-exact, applies within 1e-13
    import torch
    if case == "lap3d":
        rp, ci, v = gen.laplace3d(24)
    elif case == "diffusion2d":
        rp, ci, v, _ = gen.diffusion2d_edges(80)
    elif case == "convdiff_scrambled":
        rp, ci, v = _scrambled(*gen.convdiff2d(50, 40, peclet=10.0, shift=0.01), seed=5)
    else:
        rp, ci, v = gen.lognormal_random(4000, mu=2.0, sigma=1.0, hi=300, seed=8)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    b = gen.rhs_uniform(n, 3)
    tag = V.chow_patel_tag(sweeps, iters)
    kinds = [(V.chow_patel_ilu_precond, oracle.chow_patel_ilu)]
    if case != "lognormal":  # IC0 of a nonsymmetric matrix takes roots of negative pivots
        kinds.append((V.chow_patel_icc_precond, oracle.chow_patel_icc))
    for cls, fn in kinds:
        P = cls(A, tag)
        F = fn(rp, ci, v, sweeps)
        _check_against(P, F)
        z = _np(P.apply(torch.tensor(b, device="cuda")))
        ref = oracle.chow_patel_apply(F, b, iters)
        assert rel_err(z, ref) < 1e-13


def test_float32(V):
    # FP32 matrices: the same algorithm in single precision, within FP32 error of FP64
    import torch
    rp, ci, v = gen.convdiff2d(40, 40, peclet=5.0, shift=0.02)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v.astype(np.float32))
    b = gen.rhs_uniform(n, 4)
    P = V.chow_patel_ilu_precond(A)
    z = _np(P.apply(torch.tensor(b, dtype=torch.float32, device="cuda")))
    ref = oracle.chow_patel_apply(oracle.chow_patel_ilu(rp, ci, v, 3), b, 2)
    assert rel_err(z.astype(np.float64), ref) < 1e-5


def test_solves_golden(V, golden):
    # BiCGStab + chow_patel_ilu_precond, CG + chow_patel_icc_precond (default
    # tag) against the reference's runs
    d = golden("chow_patel.npz")
    A = V.compressed_matrix(d["cp"], d["cc"], d["cv"])
    tag = V.bicgstab_tag(1e-10, 2000)
    x = _np(V.solve(A, d["b_cd"], tag, V.chow_patel_ilu_precond(A)))
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), int(d["iters_bicgstab_cpilu"]))
    assert rel_err(x, d["x_bicgstab_cpilu"]) < 1e-6
    S = V.compressed_matrix(d["sp"], d["sc"], d["sv"])
    tag = V.cg_tag(1e-10, 2000)
    x = _np(V.solve(S, d["b_sd"], tag, V.chow_patel_icc_precond(S)))
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), int(d["iters_cg_cpicc"]))
    assert rel_err(x, d["x_cg_cpicc"]) < 1e-6


def test_solve_matches_oracle_larger(V):
    # 3D: CG with IC0 needs fewer iterations than without, like the oracle's run
    rp, ci, v = gen.laplace3d(40)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 6)
    A = V.compressed_matrix(rp, ci, v)
    tag = V.cg_tag(1e-10, 3000)
    x = _np(V.solve(A, b, tag, V.chow_patel_icc_precond(A)))
    xo, it, _ = oracle.solve("cg", rp, ci, v, b, 1e-10, 3000, "cpicc")
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), it)
    assert rel_err(x, xo) < 1e-8
    assert oracle.rel_residual(rp, ci, v, x, b) < 1e-9


def test_rejects_unsorted_and_missing_diagonal(V):
    # the reference's merges assume ascending columns and a diagonal in every row
    rp = np.array([0, 2, 4, 6], np.uint32)
    ci = np.array([1, 0, 0, 1, 1, 2], np.uint32)  # row 0 descending
    v = np.array([1.0, 4.0, 1.0, 4.0, 1.0, 4.0])
    A = V.compressed_matrix(rp, ci, v)
    with pytest.raises(V.VclgbError) as e:
        V.chow_patel_ilu_precond(A)
    assert e.value.status == V.INVALID_MATRIX
    ci = np.array([0, 1, 0, 2, 1, 2], np.uint32)  # row 1 lacks (1, 1)
    B = V.compressed_matrix(rp, ci, v)
    for cls in (V.chow_patel_ilu_precond, V.chow_patel_icc_precond):
        with pytest.raises(V.VclgbError) as e:
            cls(B)
        assert e.value.status == V.ZERO_ON_DIAGONAL
    ci = np.array([0, 1, 0, 1, 1, 2], np.uint32)
    C = V.compressed_matrix(rp, ci, np.array([4.0, 1.0, 1.0, 0.0, 1.0, 4.0]))
    with pytest.raises(V.VclgbError) as e:
        V.chow_patel_icc_precond(C)
    assert e.value.status == V.ZERO_ON_DIAGONAL


def test_diagonal_and_empty_matrices(V):
    # no off-diagonal entries: the apply divides by the scaled diagonals; an
    # empty matrix builds
    import torch
    n = 50
    rp = np.arange(n + 1, dtype=np.uint32)
    ci = np.arange(n, dtype=np.uint32)
    v = np.linspace(1.0, 5.0, n)
    A = V.compressed_matrix(rp, ci, v)
    b = gen.rhs_uniform(n, 7)
    for cls, fn in ((V.chow_patel_ilu_precond, oracle.chow_patel_ilu),
                    (V.chow_patel_icc_precond, oracle.chow_patel_icc)):
        P = cls(A)
        assert P.info().nnz_L == 0 and P.info().nnz_U == 0
        z = _np(P.apply(torch.tensor(b, device="cuda")))
        assert rel_err(z, oracle.chow_patel_apply(fn(rp, ci, v, 3), b, 2)) < 1e-15
    E = V.compressed_matrix(np.zeros(1, np.uint32), np.zeros(0, np.uint32), np.zeros(0), 0, 0)
    for cls in (V.chow_patel_ilu_precond, V.chow_patel_icc_precond):
        inf = cls(E).info()
        assert inf.nnz_L == 0 and inf.nnz_U == 0
