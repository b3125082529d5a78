"""Solvers on the GPU against the reference's golden outputs and the oracle:
same stopping rule, iteration counts within 2%, solutions within tolerance,
true FP64 relative residuals reported."""
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


@pytest.mark.parametrize("pc", ["none", "jacobi", "ilu0"])
def test_cg_golden(V, golden, pc):
    d = golden("cg_laplace2d.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    P = {"none": None, "jacobi": V.jacobi_precond(A), "ilu0": V.ilu0_precond(A)}[pc]
    tag = V.cg_tag(float(d["tol"]), int(d["max_iters"]))
    x = _np(V.solve(A, d["b"], tag, P))
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), int(d["iters_" + pc]))
    assert rel_err(x, d["x_" + pc]) < 1e-6
    assert abs(tag.error() - float(d["error_" + pc])) < 0.05 * float(d["error_" + pc])
    assert oracle.rel_residual(d["rp"], d["ci"], d["v"], x, d["b"]) < 1e-7


@pytest.mark.parametrize("pc", ["none", "jacobi"])
def test_bicgstab_golden(V, golden, pc):
    d = golden("bicgstab_convdiff.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    P = V.jacobi_precond(A) if pc == "jacobi" else None
    tag = V.bicgstab_tag(float(d["tol"]), int(d["max_iters"]))
    x = _np(V.solve(A, d["b"], tag, P))
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), int(d["iters_" + pc]))
    assert rel_err(x, d["x_" + pc]) < 1e-7


def test_gmres_against_oracle_and_reference(V, golden):
    d = golden("gmres_convdiff_1thread.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    tag = V.gmres_tag(1e-10, 600, 30)
    x = _np(V.solve(A, d["b"], tag))
    xo, it_o, err_o = oracle.solve("gmres", d["rp"], d["ci"], d["v"], d["b"], 1e-10, 600,
                                   krylov_dim=30)
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), it_o)
    assert rel_err(x, xo) < 1e-7
    # the reference host backend needs more iterations (its stage-1 defect)
    assert tag.iters() <= int(d["iters"])
    assert oracle.rel_residual(d["rp"], d["ci"], d["v"], x, d["b"]) < 2e-10


@pytest.mark.parametrize("pc", ["none", "jacobi"])
@pytest.mark.parametrize("kd", [1, 7, 45, 64])
def test_gmres_per_phase_krylov_dims(V, kd, pc):
    # 40,000 rows, above the cluster launch's limit: the per-phase GMRES and the
    # preconditioned (Householder-variant) GMRES at Krylov dimensions from 1
    # (R(0,0), xi_0 and the step's test come from the first product's epilogue
    # alone) to the largest, 64.  Dimension 1 stalls: capped at 60 iterations,
    # its status, count, error estimate and x follow the oracle's.
    import torch
    rp, ci, v = gen.convdiff2d(200, 200, peclet=5.0, shift=0.05)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 18)
    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A) if pc == "jacobi" else None
    cap = 60 if kd == 1 else 3000
    tag = V.gmres_tag(1e-10, cap, kd)
    bd = torch.tensor(b, device="cuda")
    x = _np(V.solve(A, bd, tag, P) if P else V.solve(A, bd, tag))
    xo, it_o, err_o = oracle.solve("gmres", rp, ci, v, b, 1e-10, cap, pc, krylov_dim=kd)
    if kd == 1:
        assert tag.status() == V.NOT_CONVERGED
        assert tag.iters() == it_o == cap
        assert abs(tag.error() - err_o) < 1e-6 * err_o
        assert rel_err(x, xo) < 1e-8
        return
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), it_o, 0.05), (tag.iters(), it_o)
    assert rel_err(x, xo) < 1e-7
    # the Jacobi form stops on the preconditioned residual (4e-10 true here)
    assert oracle.rel_residual(rp, ci, v, x, b) < (2e-10 if pc == "none" else 1e-9)


@pytest.mark.parametrize("pc", ["none", "jacobi"])
def test_gmres_per_phase_float32(V, pc):
    # the FP32 instantiations of both GMRES forms on 40,000 rows (above the
    # cluster launch's limit) to 1e-5: the oracle's FP64 count within 10 % and
    # the FP32 solution's true residual, evaluated in FP64, near the tolerance
    import torch
    rp, ci, v = gen.convdiff2d(200, 200, peclet=5.0, shift=0.05)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 18)
    A = V.compressed_matrix(rp, ci, v.astype(np.float32))
    P = V.jacobi_precond(A) if pc == "jacobi" else None
    tag = V.gmres_tag(1e-5, 3000, 30)
    bd = torch.tensor(b.astype(np.float32), device="cuda")
    x = _np(V.solve(A, bd, tag, P) if P else V.solve(A, bd, tag))
    assert x.dtype == np.float32
    _, it_o, _ = oracle.solve("gmres", rp, ci, v, b, 1e-5, 3000, pc, krylov_dim=30)
    assert tag.status() == V.SUCCESS
    assert abs(tag.iters() - it_o) <= max(3, int(0.1 * it_o)), (tag.iters(), it_o)
    # the Jacobi form stops on the preconditioned residual (3.8e-5 true in FP64)
    res = oracle.rel_residual(rp, ci, v, x.astype(np.float64), b)
    assert res < (1e-4 if pc == "none" else 5e-4), res


@pytest.mark.parametrize("pc", ["none", "jacobi"])
def test_bicgstab_per_phase_float32(V, pc):
    # the FP32 instantiation of the per-phase BiCGStab (40,000 rows, above the
    # cluster launch's limit) to 1e-5.  BiCGStab's count follows rounding (the
    # oracle's threaded dot products gave 47 and 49 on this input), so the
    # oracle is a sanity band; the true residual, in FP64, is the check.
    import torch
    rp, ci, v = gen.convdiff2d(200, 200, peclet=5.0, shift=0.05)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 18)
    A = V.compressed_matrix(rp, ci, v.astype(np.float32))
    P = V.jacobi_precond(A) if pc == "jacobi" else None
    tag = V.bicgstab_tag(1e-5, 3000)
    bd = torch.tensor(b.astype(np.float32), device="cuda")
    x = _np(V.solve(A, bd, tag, P) if P else V.solve(A, bd, tag))
    assert x.dtype == np.float32
    _, it_o, _ = oracle.solve("bicgstab", rp, ci, v, b, 1e-5, 3000, pc)
    assert tag.status() == V.SUCCESS
    assert abs(tag.iters() - it_o) <= 0.35 * it_o, (tag.iters(), it_o)
    res = oracle.rel_residual(rp, ci, v, x.astype(np.float64), b)
    assert res < 5e-4, res


@pytest.mark.parametrize("pc", ["jacobi", "ilu0", "row1", "cpilu"])
@pytest.mark.parametrize("kd", [30, 10])
def test_gmres_precond_golden(V, golden, pc, kd):
    # linalg::solve(A, b, gmres_tag, precond): the reference's Householder
    # variant (gmres.hpp:449-631) -- iterations within 2 %, x within 1e-8
    d = golden("gmres_precond_convdiff.npz")
    key = "%s_%d" % (pc, kd)
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    P = {"jacobi": lambda: V.jacobi_precond(A), "ilu0": lambda: V.ilu0_precond(A),
         "row1": lambda: V.row_scaling(A, V.row_scaling_tag(1)), "cpilu": lambda: V.chow_patel_ilu_precond(A)}[pc]()
    tag = V.gmres_tag(float(d["tol"]), int(d["max_iters"]), kd)
    x = _np(V.solve(A, d["b"], tag, P))
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), int(d["iters_" + key])), (tag.iters(), d["iters_" + key])
    assert rel_err(x, d["x_" + key]) < 1e-8
    assert tag.error() < float(d["tol"])
    assert oracle.rel_residual(d["rp"], d["ci"], d["v"], x, d["b"]) < 1e-8


def test_gmres_precond_iteration_cap(V, golden):
    # max_iters 25 with Krylov dimension 10: max_restarts = 1, two cycles of 10
    # steps, status NOT_CONVERGED and the reference's estimate
    d = golden("gmres_precond_convdiff.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    tag = V.gmres_tag(1e-10, 25, 10)
    V.solve(A, d["b"], tag, V.jacobi_precond(A))
    xo, it_o, err_o = oracle.solve("gmres", d["rp"], d["ci"], d["v"], d["b"], 1e-10, 25, "jacobi",
                                   krylov_dim=10)
    assert tag.status() == V.NOT_CONVERGED
    assert tag.iters() == it_o == 30
    assert abs(tag.error() - err_o) < 1e-6 * err_o


def test_mixed_cg_golden(V, golden):
    d = golden("mixed_cg_laplace2d.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    tag = V.mixed_precision_cg_tag(float(d["tol"]), int(d["max_iters"]), float(d["inner_tol"]))
    x = _np(V.solve(A, d["b"], tag))
    assert tag.status() == V.SUCCESS
    # FP32 inner products round differently on the GPU: allow 5% on iterations
    assert abs(tag.iters() - int(d["iters"])) <= max(2, 0.05 * int(d["iters"]))
    assert oracle.rel_residual(d["rp"], d["ci"], d["v"], x, d["b"]) < 1e-8


def test_refined_cg_reaches_fp64_residual(V):
    rp, ci, v, f = gen.diffusion3d(32, corr=4.0, contrast=1e4, seed=2)
    A = V.compressed_matrix(rp, ci, v)
    tag = V.refined_cg_tag(1e-10, 100000, 1e-4)
    x = _np(V.solve(A, f, tag))
    assert tag.status() == V.SUCCESS
    rr = oracle.rel_residual(rp, ci, v, x, f)
    assert rr < 1e-10 and tag.outer >= 2
    assert abs(rr - tag.error()) < 1e-3 * rr + 1e-16
    xo, outer, inner, rro = oracle.refined_cg(rp, ci, v, f, tol=1e-10, inner_tol=1e-4)
    assert rro < 1e-10
    # same algorithm, different FP32 rounding: inner totals within 15%
    assert abs(tag.iters() - inner) <= 0.15 * inner + 5


def test_refined_cg_banded_and_scrambled(V):
    # the inner copy is stored by diagonal for a banded matrix and stays CSR
    # when a scrambled numbering spreads the entries over many diagonals; both
    # reach the FP64 tolerance and agree
    rp, ci, v = gen.laplace2d(60, 50)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 8)
    p = np.random.default_rng(8).permutation(n)
    rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    r2, c2 = p[rows], p[ci.astype(np.int64)]
    order = np.lexsort((c2, r2))
    rp2 = np.zeros(n + 1, np.int64)
    np.add.at(rp2, r2 + 1, 1)
    rp2, ci2, v2 = np.cumsum(rp2).astype(np.uint32), c2[order].astype(np.uint32), v[order]
    b2 = np.empty(n)
    b2[p] = b
    xs = []
    for (R, C, W, B) in ((rp, ci, v, b), (rp2, ci2, v2, b2)):
        A = V.compressed_matrix(R, C, W)
        tag = V.refined_cg_tag(1e-10, 100000, 1e-4)
        x = _np(V.solve(A, B, tag))
        assert tag.status() == V.SUCCESS
        assert oracle.rel_residual(R, C, W, x, B) < 1e-10
        xs.append(x)
    assert rel_err(xs[1][p], xs[0]) < 1e-8


def test_reference_cpu_case_laplace256(V):
    # 256x256 Laplacian (h = 1/257), b ~ U[-1,1] seed 0, Jacobi-PCG to 1e-8, max 2000
    rp, ci, v = gen.laplace2d(256, 256, scaled=True)
    b = gen.rhs_uniform(len(rp) - 1, 0)
    A = V.compressed_matrix(rp, ci, v)
    tag = V.cg_tag(1e-8, 2000)
    x = _np(V.solve(A, b, tag, V.jacobi_precond(A)))
    xo, it_o, err_o = oracle.solve("cg", rp, ci, v, b, 1e-8, 2000, "jacobi")
    assert iters_close(tag.iters(), it_o)
    assert rel_err(x, xo) < 1e-6


@pytest.mark.parametrize("fmt", ["ell", "sell", "hyb"])
def test_pipelined_cg_other_formats(V, fmt):
    rp, ci, v = gen.laplace3d(24)
    b = gen.rhs_uniform(len(rp) - 1, 4)
    A = V.compressed_matrix(rp, ci, v)
    M = {"ell": lambda: V.ell_matrix(A), "sell": lambda: V.sliced_ell_matrix(A, 32, 1),
         "hyb": lambda: V.hyb_matrix(A)}[fmt]()
    tag = V.cg_tag(1e-10, 1000)
    x = _np(V.solve(M, b, tag))
    xo, it_o, _ = oracle.solve("cg", rp, ci, v, b, 1e-10, 1000)
    assert iters_close(tag.iters(), it_o)
    assert rel_err(x, xo) < 1e-8


def test_bicgstab_on_hyb_and_sell(V):
    rp, ci, v = gen.lognormal_random(20000, mu=2.0, sigma=0.5, hi=60, seed=7)
    b = gen.rhs_uniform(len(rp) - 1, 1)
    A = V.compressed_matrix(rp, ci, v)
    xo, it_o, _ = oracle.solve("bicgstab", rp, ci, v, b, 1e-10, 400)
    for M in (A, V.sliced_ell_matrix(A, 32, 256), V.hyb_matrix(A)):
        tag = V.bicgstab_tag(1e-10, 400)
        x = _np(V.solve(M, b, tag))
        assert tag.status() == V.SUCCESS
        assert abs(tag.iters() - it_o) <= max(2, 0.1 * it_o)
        assert oracle.rel_residual(rp, ci, v, x, b) < 1e-8


def test_float32_cg(V):
    rp, ci, v = gen.laplace2d(64)
    b = gen.rhs_uniform(len(rp) - 1, 2)
    A = V.compressed_matrix(rp, ci, v.astype(np.float32))
    tag = V.cg_tag(1e-5, 2000)
    x = _np(V.solve(A, b.astype(np.float32), tag, V.jacobi_precond(A)))
    assert tag.status() == V.SUCCESS
    assert oracle.rel_residual(rp, ci, v, x.astype(np.float64), b) < 1e-4


def test_max_iterations_status(V):
    rp, ci, v = gen.laplace2d(64)
    b = gen.rhs_uniform(len(rp) - 1, 2)
    A = V.compressed_matrix(rp, ci, v)
    tag = V.cg_tag(1e-14, 7)
    V.solve(A, b, tag)
    assert tag.status() == V.NOT_CONVERGED and tag.iters() == 7
    xo, it_o, err_o = oracle.solve("cg", rp, ci, v, b, 1e-14, 7)
    assert abs(tag.error() - err_o) < 1e-6 * err_o


def test_zero_rhs(V):
    rp, ci, v = gen.laplace2d(16)
    A = V.compressed_matrix(rp, ci, v)
    tag = V.cg_tag(1e-8, 100)
    x = _np(V.solve(A, np.zeros(len(rp) - 1), tag))
    assert tag.iters() == 0 and not x.any()


def test_invalid_matrix_rejected(V):
    rp = np.array([0, 2, 1, 3], np.uint32)  # not monotone
    with pytest.raises(V.VclgbError) as e:
        V.compressed_matrix(rp, np.array([0, 1, 2], np.uint32), np.ones(3))
    assert e.value.status == V.INVALID_MATRIX
    rp = np.array([0, 1, 2], np.uint32)
    with pytest.raises(V.VclgbError) as e:
        V.compressed_matrix(rp, np.array([0, 5], np.uint32), np.ones(2), 2, 2)
    assert e.value.status == V.INVALID_MATRIX


def test_zero_on_diagonal(V):
    rp = np.array([0, 1, 2], np.uint32)
    A = V.compressed_matrix(rp, np.array([0, 0], np.uint32), np.ones(2), 2, 2)
    with pytest.raises(V.VclgbError) as e:
        V.jacobi_precond(A)
    assert e.value.status == V.ZERO_ON_DIAGONAL


@pytest.mark.parametrize("p", [0, 1, 2])
def test_row_scaling_golden(V, golden, p):
    # row_scaling<compressed_matrix>: the row norms bit-exact (applied to a
    # vector of ones they come back as 1/norm), BiCGStab preconditioned by them
    # against the reference's run
    import torch
    d = golden("row_scaling_convdiff.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    P = V.row_scaling(A, V.row_scaling_tag(p))
    ones = torch.ones(len(d["rp"]) - 1, dtype=torch.float64, device="cuda")
    assert np.array_equal(_np(P.apply(ones)), 1.0 / d["norm%d" % p])
    tag = V.bicgstab_tag(1e-10, 2000)
    x = _np(V.solve(A, d["b"], tag, P))
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), int(d["iters_bicgstab_row%d" % p]))
    assert rel_err(x, d["x_bicgstab_row%d" % p]) < 1e-6
    if p == 2:
        L = V.compressed_matrix(d["lp"], d["lc"], d["lv"])
        tag = V.cg_tag(1e-8, 2000)
        x = _np(V.solve(L, d["lb"], tag, V.row_scaling(L, V.row_scaling_tag(2))))
        assert iters_close(tag.iters(), int(d["iters_cg_row2"]))
        assert rel_err(x, d["x_cg_row2"]) < 1e-6


def test_row_scaling_rejects_unknown_norm(V):
    rp, ci, v = gen.laplace2d(8, 8)
    A = V.compressed_matrix(rp, ci, v)
    with pytest.raises(V.VclgbError) as e:
        V.row_scaling(A, V.row_scaling_tag(3))
    assert e.value.status == V.INVALID_ARGUMENT


def test_kernel_timing_inside_captured_solves(V):
    # event pairs around each SpMV phase and vector pass, also inside the
    # solver's CUDA graphs; the solve's result does not change.  The grid is
    # above the small-system limit: below it a solve runs in one cluster
    # launch, and kernel timing (which times the per-phase kernels) keeps the
    # per-phase path
    rp, ci, v = gen.laplace2d(224, 224)
    b = gen.rhs_uniform(len(rp) - 1, 2)
    A = V.compressed_matrix(rp, ci, v)
    t0 = V.cg_tag(1e-10, 2000)
    x0 = _np(V.solve(A, b, t0))
    A.be.set_kernel_timing(True)
    try:
        t1 = V.cg_tag(1e-10, 2000)
        x1 = _np(V.solve(A, b, t1))
        spmv, vec = A.be.kernel_times(0), A.be.kernel_times(1)
    finally:
        A.be.set_kernel_timing(False)
    assert np.array_equal(x0, x1) and t0.iters() == t1.iters()
    # one SpMV and one vector pass per iteration (plus the set-up pair and the
    # launches of the last captured chunk after convergence)
    assert len(spmv) >= t1.iters() and len(vec) >= t1.iters()
    assert np.all(spmv > 0) and np.median(spmv) < 1.0
    assert len(A.be.kernel_times(0)) == 0  # read and cleared


@pytest.mark.parametrize("pc", ["none", "jacobi"])
def test_large_cg_with_vectors_held_in_l2(V, pc):
    # the 128^3 Laplacian: vectors (4-5 x 16.8 MB) and matrix (200 MB) exceed L2,
    # so the solve keeps its vectors in a persisting L2 window and works on a
    # copy of x.  The headline configuration: 536 iterations to 1e-10, as the
    # reference's algorithm on the host; the true residual at the tolerance;
    # repeated solves bit-identical
    import torch
    rp, ci, v = gen.laplace3d(128)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 1)
    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A) if pc == "jacobi" else None
    bd = torch.tensor(b, device="cuda")
    xs = []
    for _ in range(2):
        tag = V.cg_tag(1e-10, 3000)
        x = V.solve(A, bd, tag, P) if P else V.solve(A, bd, tag)
        assert tag.status() == V.SUCCESS
        assert iters_close(tag.iters(), 536), tag.iters()
        xs.append(_np(x))
    assert np.array_equal(xs[0], xs[1])
    assert oracle.rel_residual(rp, ci, v, xs[0], b) < 1e-9
