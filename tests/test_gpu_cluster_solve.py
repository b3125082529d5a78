"""CG and diagonal-preconditioned CG on small systems run in one thread-block
cluster launch (up to 32,768 rows, 2,048 a CTA); larger systems, and every solve with
kernel timing on, keep the per-phase kernels.  Checked against the oracle
(the reference's algorithms on the host): iteration counts within the solver
tolerance band and the true residual at the requested tolerance, in FP64 and
FP32, on both sides of the size limit, plus the launch count that tells the
two paths apart."""
import numpy as np
import pytest

import oracle
import vclgb_gen as gen
from conftest import iters_close

pytestmark = pytest.mark.gpu

LIMIT = 32768


@pytest.fixture(scope="module")
def V():
    import torch
    import vclgb
    torch.cuda.set_device(0)
    return vclgb


@pytest.mark.parametrize("N", [20, 70, 150, 181, 182])
@pytest.mark.parametrize("pc", ["none", "jacobi"])
def test_small_cg_matches_oracle(V, N, pc):
    import torch
    rp, ci, v = gen.laplace2d(N, N)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 11)
    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A) if pc == "jacobi" else None
    tag = V.cg_tag(1e-10, 3000)
    l0 = A.be.launches()
    x = V.solve(A, torch.tensor(b, device="cuda"), tag, P) if P else \
        V.solve(A, torch.tensor(b, device="cuda"), tag)
    launches = A.be.launches() - l0
    xs = x.cpu().numpy()
    _, it_ref, _ = oracle.solve("cg", rp, ci, v, b, 1e-10, 3000, pc)
    assert tag.status() == V.SUCCESS
    assert iters_close(tag.iters(), it_ref), (tag.iters(), it_ref)
    assert oracle.rel_residual(rp, ci, v, xs, b) < 1e-9
    if n <= LIMIT:
        assert launches <= 4, launches  # one cluster launch (plus the state set-up)
    else:
        assert launches > tag.iters(), launches


@pytest.mark.parametrize("pc", ["none", "jacobi"])
def test_small_cg_fp32(V, pc):
    import torch
    rp, ci, v = gen.laplace2d(60, 60)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 12)
    A = V.compressed_matrix(rp, ci, v.astype(np.float32))
    P = V.jacobi_precond(A) if pc == "jacobi" else None
    tag = V.cg_tag(1e-5, 3000)
    bd = torch.tensor(b.astype(np.float32), device="cuda")
    x = V.solve(A, bd, tag, P) if P else V.solve(A, bd, tag)
    _, it_ref, _ = oracle.solve("cg", rp, ci, v, b, 1e-5, 3000, pc)
    assert tag.status() == V.SUCCESS
    assert abs(tag.iters() - it_ref) <= max(3, it_ref // 5), (tag.iters(), it_ref)
    assert oracle.rel_residual(rp, ci, v, x.cpu().numpy().astype(np.float64), b) < 1e-4


def test_cluster_and_per_phase_paths_agree(V):
    # the same solve through the cluster path and, with kernel timing on,
    # through the per-phase kernels: equal iteration counts, solutions within
    # the solver tolerance
    import torch
    rp, ci, v = gen.laplace2d(90, 90)
    b = torch.tensor(gen.rhs_uniform(len(rp) - 1, 13), device="cuda")
    A = V.compressed_matrix(rp, ci, v)
    t0 = V.cg_tag(1e-12, 3000)
    x0 = V.solve(A, b, t0).cpu().numpy()
    A.be.set_kernel_timing(True)
    try:
        t1 = V.cg_tag(1e-12, 3000)
        x1 = V.solve(A, b, t1).cpu().numpy()
    finally:
        A.be.set_kernel_timing(False)
    assert iters_close(t0.iters(), t1.iters())
    assert np.linalg.norm(x0 - x1) / np.linalg.norm(x1) < 1e-9


@pytest.mark.parametrize("N", [30, 90, 150, 181, 182])
@pytest.mark.parametrize("pc", ["none", "jacobi"])
def test_small_bicgstab_matches_oracle(V, N, pc):
    # nonsymmetric upwind convection-diffusion; pipelined BiCGStab without a
    # preconditioner, the restarted preconditioned form with Jacobi; the
    # cluster path below the limit, per-phase above
    import torch
    rp, ci, v = gen.convdiff2d(N, N, peclet=5.0, shift=0.05)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 14)
    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A) if pc == "jacobi" else None
    tag = V.bicgstab_tag(1e-10, 3000)
    l0 = A.be.launches()
    bd = torch.tensor(b, device="cuda")
    x = V.solve(A, bd, tag, P) if P else V.solve(A, bd, tag)
    launches = A.be.launches() - l0
    _, it_ref, _ = oracle.solve("bicgstab", rp, ci, v, b, 1e-10, 3000, pc)
    assert tag.status() == V.SUCCESS
    # BiCGStab's recurrences amplify rounding differences: the iteration band
    # of the other BiCGStab parity tests
    assert abs(tag.iters() - it_ref) <= max(2, int(0.15 * it_ref)), (tag.iters(), it_ref)
    assert oracle.rel_residual(rp, ci, v, x.cpu().numpy(), b) < 1e-8
    if n <= LIMIT:
        assert launches <= 4, launches
    else:
        assert launches > tag.iters(), launches


def _random_dominant(n, per_row, seed, symmetric):
    # random pattern, up to 2 per_row off-diagonals a row spread over all
    # columns (gathers cross CTAs), dominant diagonal
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(seed)
    r = np.repeat(np.arange(n), per_row)
    c = rng.integers(0, n, n * per_row)
    M = sp.coo_matrix((rng.uniform(-1, 1, n * per_row), (r, c)), shape=(n, n)).tocsr()
    M = M + M.T if symmetric else M + sp.coo_matrix(
        (rng.uniform(-1, 1, n * per_row), (c, r)), shape=(n, n)).tocsr()
    M = M + sp.diags(np.asarray(abs(M).sum(axis=1)).ravel() + 0.5)
    M = M.tocsr()
    M.sum_duplicates()
    M.sort_indices()
    return M.indptr.astype(np.uint32), M.indices.astype(np.uint32), M.data.astype(np.float64)


@pytest.mark.parametrize("solver,pc", [("cg", "none"), ("cg", "jacobi"),
                                       ("bicgstab", "none"), ("bicgstab", "jacobi")])
def test_small_random_matrices(V, solver, pc):
    import torch
    rp, ci, v = _random_dominant(9000, 10, seed=21, symmetric=(solver == "cg"))
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 15)
    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A) if pc == "jacobi" else None
    tag = V.cg_tag(1e-10, 3000) if solver == "cg" else V.bicgstab_tag(1e-10, 3000)
    bd = torch.tensor(b, device="cuda")
    l0 = A.be.launches()
    x = V.solve(A, bd, tag, P) if P else V.solve(A, bd, tag)
    assert A.be.launches() - l0 <= 4  # the cluster path
    _, it_ref, _ = oracle.solve(solver, rp, ci, v, b, 1e-10, 3000, pc)
    assert tag.status() == V.SUCCESS
    band = 0.02 if solver == "cg" else 0.15
    assert abs(tag.iters() - it_ref) <= max(2, int(band * it_ref)), (tag.iters(), it_ref)
    assert oracle.rel_residual(rp, ci, v, x.cpu().numpy(), b) < 1e-8


@pytest.mark.parametrize("N,kd", [(30, 10), (70, 20), (70, 30), (90, 30)])
def test_small_gmres_matches_oracle(V, N, kd):
    # unpreconditioned GMRES on upwind convection-diffusion in one cluster
    # launch (x, r and the Krylov basis in shared memory): the oracle's
    # iteration count within the GMRES band, the true residual at the tolerance
    import torch
    rp, ci, v = gen.convdiff2d(N, N, peclet=5.0, shift=0.05)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 16)
    A = V.compressed_matrix(rp, ci, v)
    tag = V.gmres_tag(1e-10, 3000, kd)
    l0 = A.be.launches()
    x = V.solve(A, torch.tensor(b, device="cuda"), tag)
    launches = A.be.launches() - l0
    _, it_ref, _ = oracle.solve("gmres", rp, ci, v, b, 1e-10, 3000, krylov_dim=kd)
    assert tag.status() == V.SUCCESS
    assert launches <= 4, launches
    assert iters_close(tag.iters(), it_ref, 0.05), (tag.iters(), it_ref)
    assert oracle.rel_residual(rp, ci, v, x.cpu().numpy(), b) < 1e-9


def test_small_gmres_fp32_and_paths_agree(V):
    import torch
    rp, ci, v = gen.convdiff2d(60, 60, peclet=5.0, shift=0.05)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 17)
    # FP32
    A32 = V.compressed_matrix(rp, ci, v.astype(np.float32))
    t32 = V.gmres_tag(1e-5, 3000, 20)
    x32 = V.solve(A32, torch.tensor(b.astype(np.float32), device="cuda"), t32)
    assert t32.status() == V.SUCCESS
    assert oracle.rel_residual(rp, ci, v, x32.cpu().numpy().astype(np.float64), b) < 1e-4
    # the cluster path and, with kernel timing on, the per-phase kernels
    A = V.compressed_matrix(rp, ci, v)
    bd = torch.tensor(b, device="cuda")
    t0 = V.gmres_tag(1e-12, 3000, 20)
    x0 = V.solve(A, bd, t0).cpu().numpy()
    A.be.set_kernel_timing(True)
    try:
        t1 = V.gmres_tag(1e-12, 3000, 20)
        x1 = V.solve(A, bd, t1).cpu().numpy()
        # a capped solve: the iteration count and status follow the same rule
        c1 = V.gmres_tag(1e-12, 25, 10)
        V.solve(A, bd, c1)
    finally:
        A.be.set_kernel_timing(False)
    assert iters_close(t0.iters(), t1.iters())
    assert np.linalg.norm(x0 - x1) / np.linalg.norm(x1) < 1e-9
    c0 = V.gmres_tag(1e-12, 25, 10)
    V.solve(A, bd, c0)
    assert c0.status() == c1.status() == V.NOT_CONVERGED
    assert c0.iters() == c1.iters()
    assert abs(c0.error() - c1.error()) < 1e-6 * c1.error()
