"""Adjoint (backward) solve: the transpose map against the oracle, gradients
against the reference host backend's own transpose solve (golden fixtures),
and against central finite differences along 64 seeded random directions."""
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


def test_transpose_map(V):
    import torch
    rp, ci, v = gen.lognormal_random(5000, mu=2.0, sigma=1.0, hi=300, seed=3)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    trp, tci, tv, mp = oracle.transpose(n, n, rp, ci, v)
    nnz = len(v)
    assert np.array_equal(_u32(V.transpose_export(A, 0, n + 1, torch.int32)), trp)
    assert np.array_equal(_u32(V.transpose_export(A, 1, nnz, torch.int32)), tci)
    assert np.array_equal(V.transpose_export(A, 2, nnz, torch.float64).cpu().numpy(), tv)
    assert np.array_equal(_u32(V.transpose_export(A, 3, nnz, torch.int32)), mp)


def test_golden_nonsymmetric_gmres_adjoint(V, golden):
    d = golden("adjoint_convdiff.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    tag = V.gmres_tag(1e-13, 3000, 30)
    x = V.solve(A, d["b"], tag)
    assert rel_err(x.cpu().numpy(), d["x"]) < 1e-9
    atag = V.gmres_tag(1e-13, 3000, 30)
    lam, gA = V.solve_adjoint(A, x, x - V._dev(d["xt"], x.dtype), atag, solver="gmres")
    assert rel_err(lam.cpu().numpy(), d["lam"]) < 1e-8
    assert rel_err(gA.cpu().numpy(), d["dLdA"]) < 1e-8


def test_golden_spd_cg_adjoint(V, golden):
    d = golden("adjoint_diffusion2d.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    P = V.jacobi_precond(A)
    x = V.solve(A, d["b"], V.cg_tag(1e-13, 5000), P)
    lam, gA = V.solve_adjoint(A, x, x - V._dev(d["xt"], x.dtype), V.cg_tag(1e-13, 5000),
                              solver="cg", precond=P, symmetric=True)
    assert rel_err(lam.cpu().numpy(), d["lam"]) < 1e-9
    assert rel_err(gA.cpu().numpy(), d["dLdA"]) < 1e-9


def _assemble_kappa(N, kx, ky):
    """Matrix values of the 2D edge-coefficient diffusion operator and the
    per-entry derivative map d(values)/d(kappa_e) as (entry, edge, sign)."""
    rp, ci, v = gen._fv_diffusion(np.ones((N, N)), [kx, ky])
    return rp, ci, v


@pytest.mark.parametrize("N", [48, 512])
def test_finite_differences_spd_64_directions(V, N):
    # N = 512: the configured 512^2 diffusion problem (262,144 unknowns,
    # per-edge lognormal kappa with contrast 1e3, seed 4)
    import torch
    rp, ci, v, (kx, ky) = gen.diffusion2d_edges(N, contrast=1e3, seed=4)
    n = len(rp) - 1
    rng = np.random.default_rng(77)
    b = rng.uniform(-1, 1, n)
    xt = rng.uniform(0, 1, n)

    def loss(vals, bb):
        A = V.compressed_matrix(rp, ci, vals)
        x = V.solve(A, bb, V.cg_tag(1e-13, 20000), V.jacobi_precond(A)).cpu().numpy()
        return 0.5 * np.sum((x - xt) ** 2)

    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A)
    x = V.solve(A, b, V.cg_tag(1e-13, 20000), P)
    lam, gA = V.solve_adjoint(A, x, x - V._dev(xt, torch.float64), V.cg_tag(1e-13, 20000),
                              solver="cg", precond=P, symmetric=True)
    lam, gA = lam.cpu().numpy(), gA.cpu().numpy()
    worst = 0.0
    for d in range(64):
        rd = np.random.default_rng(1000 + d)
        if d % 2 == 0:
            # direction in b: L is quadratic in b, so a large step is exact
            db = rd.standard_normal(n)
            eps = 0.5
            fd = (loss(v, b + eps * db) - loss(v, b - eps * db)) / (2 * eps)
            an = lam @ db
        else:
            # direction in the edge coefficients kappa, chained through the
            # assembly: the matrix values are affine in kappa, so
            # dA = (A(k + e dk) - A(k - e dk)) / 2e exactly and dL/dk . dk = dL/dA . dA
            dkx = rd.standard_normal(kx.shape) * kx
            dky = rd.standard_normal(ky.shape) * ky
            eps = 1e-4
            _, _, vp = _assemble_kappa(N, kx + eps * dkx, ky + eps * dky)
            _, _, vm = _assemble_kappa(N, kx - eps * dkx, ky - eps * dky)
            fd = (loss(vp, b) - loss(vm, b)) / (2 * eps)
            an = gA @ ((vp - vm) / (2 * eps))
        worst = max(worst, abs(fd - an) / max(abs(an), 1e-30))
    assert worst < 1e-6, worst


def test_finite_differences_nonsymmetric_gmres(V):
    import torch
    rp, ci, v = gen.convdiff2d(24, 22, peclet=15.0, shift=0.1)
    n = len(rp) - 1
    rng = np.random.default_rng(5)
    b = rng.uniform(-1, 1, n)
    xt = rng.uniform(0, 1, n)

    def loss(vals, bb):
        A = V.compressed_matrix(rp, ci, vals)
        x = V.solve(A, bb, V.gmres_tag(1e-14, 4000, 30)).cpu().numpy()
        return 0.5 * np.sum((x - xt) ** 2)

    A = V.compressed_matrix(rp, ci, v)
    x = V.solve(A, b, V.gmres_tag(1e-14, 4000, 30))
    lam, gA = V.solve_adjoint(A, x, x - V._dev(xt, torch.float64), V.gmres_tag(1e-14, 4000, 30),
                              solver="gmres")
    lam, gA = lam.cpu().numpy(), gA.cpu().numpy()
    worst = 0.0
    for d in range(16):
        rd = np.random.default_rng(2000 + d)
        if d % 2 == 0:
            db = rd.standard_normal(n)
            eps = 0.5
            fd = (loss(v, b + eps * db) - loss(v, b - eps * db)) / (2 * eps)
            an = lam @ db
        else:
            dA = rd.standard_normal(len(v)) * np.abs(v)
            eps = 1e-5
            fd = (loss(v + eps * dA, b) - loss(v - eps * dA, b)) / (2 * eps)
            an = gA @ dA
        worst = max(worst, abs(fd - an) / max(abs(an), 1e-30))
    assert worst < 1e-6, worst
