"""GPU conversions CSR -> ELL / SELL-C-sigma / HYB / COO: bit-exact against the
reference's copy() output (golden) and the oracle, plus SpMV per format."""
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


def _ell_arrays(M, n):
    import torch
    inf = M.info()
    w = inf.ell_width
    return w, _u32(M.export(0, n * w, torch.int32)), M.export(1, n * w, torch.float64).cpu().numpy()


def test_coo_golden(V, golden):
    # coordinate_matrix arrays and group boundaries bit-exact against the
    # reference's copy(); the product against the reference's host product
    import torch
    d = golden("coo_lognormal.npz")
    rp, ci, v, ncols = d["rp"], d["ci"], d["v"], int(d["ncols"])
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v, n, ncols)
    Co = V.coordinate_matrix(A)
    inf = Co.info()
    assert inf.format == V.COO and inf.nnz == int(d["nnz"][0]) and inf.stored == int(d["nnz"][1])
    assert np.array_equal(_u32(Co.export(0, 2 * inf.stored, torch.int32)), d["coords"])
    assert np.array_equal(Co.export(1, inf.stored, torch.float64).cpu().numpy(), d["elems"])
    assert np.array_equal(_u32(Co.export(2, 65, torch.int32)), d["groups"])
    y = torch.tensor(d["y0"], device="cuda")
    V.prod(Co, d["x"], alpha=float(d["alpha"]), y=y, beta=float(d["beta"]))
    assert rel_err(y.cpu().numpy(), d["y"]) < 1e-13
    # the same arrays wrapped as the reference's own buffers
    W = V.wrap_coordinate(n, ncols, inf.nnz, Co.export(0, 2 * inf.nnz, torch.int32),
                          Co.export(1, inf.nnz, torch.float64))
    assert np.array_equal(_u32(W.export(2, 65, torch.int32)), d["groups"])
    y2 = torch.tensor(d["y0"], device="cuda")
    V.prod(W, d["x"], alpha=float(d["alpha"]), y=y2, beta=float(d["beta"]))
    assert np.array_equal(y2.cpu().numpy(), y.cpu().numpy())


@pytest.mark.parametrize("case", ["lognormal", "laplace3d", "empty_rows"])
def test_coo_spmv_shapes(V, case):
    # long rows across many warp chunks, short stencil rows, empty rows
    if case == "lognormal":
        rp, ci, v = gen.lognormal_random(30000, mu=2.5, sigma=1.2, hi=2000, seed=9)
    elif case == "laplace3d":
        rp, ci, v = gen.laplace3d(30)
    else:
        rp0, ci, v = gen.lognormal_random(5000, mu=1.0, sigma=1.0, hi=40, seed=3)
        keep = np.random.default_rng(3).uniform(size=5000) < 0.5
        lens = np.diff(rp0.astype(np.int64)) * keep
        mask = np.repeat(keep, np.diff(rp0.astype(np.int64)))
        ci, v = ci[mask], v[mask]
        rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint32)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    Co = V.coordinate_matrix(A)
    x = np.random.default_rng(4).uniform(-1, 1, n)
    y0 = np.random.default_rng(5).uniform(-1, 1, n)
    import torch
    for alpha, beta in ((1.0, 0.0), (-0.75, 2.0)):
        y = torch.tensor(y0, device="cuda")
        V.prod(Co, x, alpha=alpha, y=y, beta=beta)
        assert rel_err(y.cpu().numpy(), oracle.spmv(rp, ci, v, x, alpha, beta, y0)) < 1e-13


def test_coo_wrap_rejects_unsorted_rows(V):
    import torch
    coords = torch.tensor(np.array([1, 0, 0, 1], np.uint32).view(np.int32), device="cuda")
    with pytest.raises(V.VclgbError) as e:
        V.wrap_coordinate(2, 2, 2, coords, torch.ones(2, dtype=torch.float64, device="cuda"))
    assert e.value.status == V.INVALID_MATRIX


@pytest.mark.parametrize("name", ["formats_lognormal.npz", "formats_laplace2d.npz"])
def test_golden_conversions(V, golden, name):
    import torch
    d = golden(name)
    rp, ci, v, x = d["rp"], d["ci"], d["v"], d["x"]
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    E = V.ell_matrix(A)
    w, coords, elems = _ell_arrays(E, n)
    assert w == int(d["ell_width"][0])
    assert np.array_equal(coords, d["ell_coords"]) and np.array_equal(elems, d["ell_elems"])
    S = V.sliced_ell_matrix(A, int(d["C"]), 1)
    inf = S.info()
    assert np.array_equal(_u32(S.export(0, inf.num_slices, torch.int32)), d["sell_cpb"])
    assert np.array_equal(_u32(S.export(2, inf.num_slices, torch.int32)), d["sell_bs"])
    assert np.array_equal(_u32(S.export(1, inf.stored, torch.int32)), d["sell_cols"])
    assert np.array_equal(S.export(3, inf.stored, torch.float64).cpu().numpy(), d["sell_elems"])
    H = V.hyb_matrix(A, float(d["threshold"]))
    hi = H.info()
    assert hi.ell_width == int(d["hyb_width"][0]) and hi.tail_nnz == int(d["hyb_tail_nnz"][0])
    assert np.array_equal(_u32(H.export(0, n * hi.ell_width, torch.int32)), d["hyb_ell_coords"])
    assert np.array_equal(H.export(1, n * hi.ell_width, torch.float64).cpu().numpy(),
                          d["hyb_ell_elems"])
    assert np.array_equal(_u32(H.export(2, n + 1, torch.int32)), d["hyb_tail_rp"])
    assert np.array_equal(_u32(H.export(3, hi.tail_nnz, torch.int32)), d["hyb_tail_ci"])
    assert np.array_equal(H.export(4, hi.tail_nnz, torch.float64).cpu().numpy(), d["hyb_tail_v"])
    for M, key in ((E, "y_ell"), (S, "y_sell"), (H, "y_hyb")):
        if key in d:
            assert rel_err(V.prod(M, x).cpu().numpy(), d[key]) < 1e-13, key


def test_hyb_float_threshold(V, golden):
    d = golden("hyb_f32_laplace2d.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"].astype(np.float32))
    assert V.hyb_matrix(A, 0.8).info().ell_width == int(d["width"][0])


@pytest.mark.parametrize("sigma", [1, 8, 256])
@pytest.mark.parametrize("C", [32, 64, 7])
def test_sell_sigma_against_oracle(V, C, sigma):
    import torch
    rp, ci, v = gen.lognormal_random(20000, mu=2.0, sigma=1.0, hi=300, seed=5)
    n = len(rp) - 1
    ref = oracle.sell(rp, ci, v, C=C, sigma=sigma)
    A = V.compressed_matrix(rp, ci, v)
    S = V.sliced_ell_matrix(A, C, sigma)
    inf = S.info()
    assert inf.stored == ref["cols"].size
    assert np.array_equal(_u32(S.export(4, n, torch.int32)), ref["perm"])
    assert np.array_equal(_u32(S.export(0, inf.num_slices, torch.int32)), ref["cpb"])
    assert np.array_equal(_u32(S.export(2, inf.num_slices, torch.int32)), ref["bs"])
    assert np.array_equal(_u32(S.export(1, inf.stored, torch.int32)), ref["cols"])
    assert np.array_equal(S.export(3, inf.stored, torch.float64).cpu().numpy(), ref["elems"])
    x = np.random.default_rng(2).uniform(-1, 1, n)
    assert rel_err(V.prod(S, x).cpu().numpy(), oracle.spmv(rp, ci, v, x)) < 1e-13
    if sigma > 1:  # sorting windows shrink the padding
        assert inf.stored <= oracle.sell(rp, ci, v, C=C, sigma=1)["cols"].size


@pytest.mark.parametrize("thr", [0.5, 0.8, 0.95, 1.0])
def test_hyb_tail_segments(V, thr):
    # long tails spanning many warp chunks exercise the segmented reduction
    rp, ci, v = gen.lognormal_random(30000, mu=2.5, sigma=1.2, hi=2000, seed=9)
    n = len(rp) - 1
    ref = oracle.hyb(rp, ci, v, n, thr)
    A = V.compressed_matrix(rp, ci, v)
    H = V.hyb_matrix(A, thr)
    hi = H.info()
    assert hi.ell_width == ref["width"]
    assert hi.tail_nnz == max(ref["tail_nnz"], 1)
    x = np.random.default_rng(4).uniform(-1, 1, n)
    y0 = np.random.default_rng(5).uniform(-1, 1, n)
    import torch
    y = torch.tensor(y0, device="cuda")
    V.prod(H, x, alpha=-0.75, y=y, beta=2.0)
    assert rel_err(y.cpu().numpy(), oracle.spmv(rp, ci, v, x, -0.75, 2.0, y0)) < 1e-13


def test_ell_float32(V):
    rp, ci, v = gen.laplace3d(20)
    A = V.compressed_matrix(rp, ci, v.astype(np.float32))
    x = np.random.default_rng(3).uniform(-1, 1, len(rp) - 1).astype(np.float32)
    for M in (V.ell_matrix(A), V.sliced_ell_matrix(A, 32, 1), V.hyb_matrix(A)):
        assert rel_err(V.prod(M, x).cpu().numpy(), oracle.spmv(rp, ci, v, x)) < 1e-5


def test_full_size_lognormal_formats(V):
    # 1M-row lognormal matrix: all formats agree with the oracle (size-independent check)
    rp, ci, v = gen.lognormal_random(1 << 20, seed=1)
    n = len(rp) - 1
    x = np.random.default_rng(1).uniform(-1, 1, n)
    ref = oracle.spmv(rp, ci, v, x)
    A = V.compressed_matrix(rp, ci, v)
    for M in (A, V.sliced_ell_matrix(A, 32, 256), V.hyb_matrix(A)):
        assert rel_err(V.prod(M, x).cpu().numpy(), ref) < 1e-13


def _same_nonfinite(out, ref):
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(out), fin)
    assert np.array_equal(out[~fin], ref[~fin], equal_nan=True)
    assert rel_err(out[fin], ref[fin]) < 1e-13


def test_padded_formats_skip_stored_zeros(V):
    # Stored zeros (ELL/SELL padding and explicit zeros) contribute nothing,
    # as in the reference ELL and SELL kernels, even when x holds inf/NaN there:
    # x[0] = inf reaches every padding slot (column 0), x[n] = NaN is hit only
    # through explicit zeros appended to every 7th row.
    rp, ci, v = gen.laplace2d(30, 23)
    n = len(rp) - 1
    lens = np.diff(rp)
    extra = (np.arange(n) % 7 == 3).astype(np.int64)
    rp2 = np.concatenate([[0], np.cumsum(lens + extra)]).astype(rp.dtype)
    ci2 = np.empty(rp2[-1], dtype=ci.dtype)
    v2 = np.empty(rp2[-1])
    for r in range(n):
        ci2[rp2[r]:rp2[r] + lens[r]] = ci[rp[r]:rp[r + 1]]
        v2[rp2[r]:rp2[r] + lens[r]] = v[rp[r]:rp[r + 1]]
        if extra[r]:
            ci2[rp2[r + 1] - 1] = n
            v2[rp2[r + 1] - 1] = 0.0
    x = np.random.default_rng(8).uniform(-1, 1, n + 1)
    x[0] = np.inf
    x[n] = np.nan
    ref = oracle.spmv(rp, ci, v, x)  # the same matrix without its explicit zeros
    assert np.isinf(ref[0]) and np.isfinite(ref[n // 2])
    A = V.compressed_matrix(rp2, ci2, v2, n, n + 1)
    for M in (V.ell_matrix(A), V.sliced_ell_matrix(A, 32, 1), V.sliced_ell_matrix(A, 7, 8),
              V.hyb_matrix(A, 1.0)):
        _same_nonfinite(V.prod(M, x).cpu().numpy(), ref)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_wrap_reference_layout(V, dtype):
    # Buffers in the reference's ell/sliced_ell/hyb layout (exported from our
    # conversions, which match the reference's copy() bit for bit) wrapped
    # without copying give the same product as the converted matrices.
    import torch
    tdt = getattr(torch, dtype)
    rp, ci, v = gen.lognormal_random(30000, mu=2.0, sigma=1.0, hi=400, seed=12)
    n = len(rp) - 1
    v = v.astype(np.float32) if dtype == "float32" else v
    A = V.compressed_matrix(rp, ci, v)
    x = np.random.default_rng(6).uniform(-1, 1, n).astype(v.dtype)
    tol = 1e-5 if dtype == "float32" else 1e-13

    E = V.ell_matrix(A)
    w = E.info().ell_width
    We = V.wrap_ell(n, n, w, E.export(0, n * w, torch.int32), E.export(1, n * w, tdt))
    assert We.info().ell_width == w and We.info().format == V.ELL

    S = V.sliced_ell_matrix(A, 32, 1)
    si = S.info()
    Ws = V.wrap_sliced_ell(n, n, 32, S.export(0, si.num_slices, torch.int32),
                           S.export(1, si.stored, torch.int32),
                           S.export(2, si.num_slices, torch.int32), S.export(3, si.stored, tdt))
    assert Ws.info().stored == si.stored and Ws.info().num_slices == si.num_slices

    H = V.hyb_matrix(A, 0.8)
    hi = H.info()
    trp = H.export(2, n + 1, torch.int32)
    tnnz = int(_u32(trp)[-1])
    assert tnnz > 0
    Wh = V.wrap_hyb(n, n, hi.ell_width, H.export(0, n * hi.ell_width, torch.int32),
                    H.export(1, n * hi.ell_width, tdt), trp, H.export(3, tnnz, torch.int32),
                    H.export(4, tnnz, tdt))
    ref = oracle.spmv(rp, ci, v, x)
    for M, W in ((E, We), (S, Ws), (H, Wh)):
        y = V.prod(M, x).cpu().numpy()
        yw = V.prod(W, x).cpu().numpy()
        assert np.array_equal(y, yw)
        assert rel_err(yw, ref) < tol
    # a solver runs on a wrapped matrix as on a converted one
    if dtype == "float64":
        rp2, ci2, v2 = gen.laplace2d(64, 64)
        n2 = len(rp2) - 1
        A2 = V.compressed_matrix(rp2, ci2, v2)
        S2 = V.sliced_ell_matrix(A2, 32, 1)
        s2 = S2.info()
        W2 = V.wrap_sliced_ell(n2, n2, 32, S2.export(0, s2.num_slices, torch.int32),
                               S2.export(1, s2.stored, torch.int32),
                               S2.export(2, s2.num_slices, torch.int32),
                               S2.export(3, s2.stored, torch.float64))
        b = np.ones(n2)
        tag = V.cg_tag(tol=1e-10, max_iterations=1000)
        x2 = V.solve(W2, b, tag).cpu().numpy()
        assert rel_err(oracle.spmv(rp2, ci2, v2, x2), b) < 1e-9


def test_coo_in_the_solvers(V):
    # the pipelined CG and BiCGStab run on a coordinate_matrix through the same
    # fused epilogues as on CSR; iterations and solutions agree
    rp, ci, v = gen.laplace2d(48, 40)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 6)
    A = V.compressed_matrix(rp, ci, v)
    Co = V.coordinate_matrix(A)
    for name, tagf in (("cg", lambda: V.cg_tag(1e-10, 3000)),
                       ("bicgstab", lambda: V.bicgstab_tag(1e-10, 3000))):
        t1, t2 = tagf(), tagf()
        x1 = V.solve(A, b, t1).cpu().numpy()
        x2 = V.solve(Co, b, t2).cpu().numpy()
        assert t2.status() == V.SUCCESS
        # CG: within 2 %; pipelined BiCGStab's stopping estimate cancels near
        # convergence, so the COO summation order moves it by a few iterations
        band = 0.02 if name == "cg" else 0.15
        assert abs(t1.iters() - t2.iters()) <= max(1, int(band * t1.iters()))
        assert rel_err(x2, x1) < 1e-7
        if name == "cg":  # pipelined BiCGStab returns before its last update
            assert oracle.rel_residual(rp, ci, v, x2, b) < 1e-9


def _sym_permute_np(rp, ci, v, p):
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    r2, c2 = p[rows], p[ci.astype(np.int64)]
    order = np.lexsort((c2, r2))
    rp2 = np.zeros(n + 1, np.int64)
    np.add.at(rp2, r2 + 1, 1)
    return np.cumsum(rp2).astype(np.uint32), c2[order].astype(np.uint32), v[order]


@pytest.mark.parametrize("key,tag", [("cm", None), ("acm_a0_g1", (0.0, 1)), ("acm_a05_g2", (0.5, 2))])
def test_cuthill_mckee_golden(V, golden, key, tag):
    # the reference's permutation exactly; P A P^T on the device equals the
    # host-built one; its bandwidth is the reference's
    import torch
    d = golden("cuthill_mckee.npz")
    rp, ci, v = d["rp"], d["ci"], d["v"]
    A = V.compressed_matrix(rp, ci, v)
    t = V.cuthill_mckee_tag() if tag is None else V.advanced_cuthill_mckee_tag(*tag)
    perm = V.reorder(A, t).cpu().numpy().view(np.uint32)
    assert np.array_equal(perm, d["perm_" + key])
    B = V.permute(A, perm)
    n = len(rp) - 1
    inf = B.info()
    brp = B.export(0, n + 1, torch.int32).cpu().numpy().view(np.uint32)
    bci = B.export(1, inf.nnz, torch.int32).cpu().numpy().view(np.uint32)
    bv = B.export(2, inf.nnz, torch.float64).cpu().numpy()
    erp, eci, ev = _sym_permute_np(rp, ci, v, perm.astype(np.int64))
    assert np.array_equal(brp, erp) and np.array_equal(bci, eci) and np.array_equal(bv, ev)
    assert V.bandwidth(A) == int(d["bw_" + key][0]) and V.bandwidth(B) == int(d["bw_" + key][1])
    # B (P x) = P (A x)
    x = np.random.default_rng(3).uniform(-1, 1, n)
    px = np.empty(n)
    px[perm] = x
    y = V.prod(A, x).cpu().numpy()
    py = np.empty(n)
    py[perm] = y
    assert rel_err(V.prod(B, px).cpu().numpy(), py) < 1e-14


def test_cuthill_mckee_ordering_in_an_ilu0_solve(V, golden):
    # the reordered system is the same system: ILU0-BiCGStab on P A P^T solves
    # A x = b (banded order: ILU0 on it drops less fill than on a scrambled one)
    d = golden("cuthill_mckee.npz")
    cp, cc, cv = d["cp"], d["cc"], d["cv"]
    A = V.compressed_matrix(cp, cc, cv)
    perm = V.reorder(A, V.cuthill_mckee_tag()).cpu().numpy().view(np.uint32)
    assert np.array_equal(perm, d["perm_cd"])
    B = V.permute(A, perm)
    assert V.bandwidth(B) == int(d["bw_cd"][1]) < V.bandwidth(A)
    n = len(cp) - 1
    b = gen.rhs_uniform(n, 9)
    pb = np.empty(n)
    pb[perm] = b
    tA, tB = V.bicgstab_tag(1e-10, 2000), V.bicgstab_tag(1e-10, 2000)
    xa = V.solve(A, b, tA, V.ilu0_precond(A)).cpu().numpy()
    xb = V.solve(B, pb, tB, V.ilu0_precond(B)).cpu().numpy()
    assert tA.status() == V.SUCCESS and tB.status() == V.SUCCESS
    assert rel_err(xb[perm], xa) < 1e-7
    assert tB.iters() <= tA.iters()


def test_permute_rejects_a_non_permutation(V):
    rp, ci, v = gen.laplace2d(5, 5)
    A = V.compressed_matrix(rp, ci, v)
    with pytest.raises(V.VclgbError) as e:
        V.permute(A, np.zeros(25, np.uint32))
    assert e.value.status == V.INVALID_ARGUMENT


def test_coo_without_entries(V):
    # an all-empty pattern: no stored entries, groups all zero, y = beta * y
    import torch
    n = 40
    A = V.compressed_matrix(np.zeros(n + 1, np.uint32), np.zeros(0, np.uint32), np.zeros(0), n, n)
    Co = V.coordinate_matrix(A)
    inf = Co.info()
    assert inf.nnz == 0 and inf.stored == 0
    assert np.array_equal(Co.export(2, 65, torch.int32).cpu().numpy(), np.zeros(65, np.int32))
    y0 = np.random.default_rng(1).uniform(-1, 1, n)
    y = torch.tensor(y0, device="cuda")
    V.prod(Co, np.ones(n), alpha=2.0, y=y, beta=-0.5)
    assert np.array_equal(y.cpu().numpy(), -0.5 * y0)
    y = torch.tensor(y0, device="cuda")
    V.prod(Co, np.ones(n), y=y)
    assert not y.cpu().numpy().any()
