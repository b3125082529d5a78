"""CSR SpMV on the GPU (adaptive kernel, row-length bins) against the oracle
and the reference's golden outputs; FP64 within 1e-13 relative 2-norm."""
import numpy as np
import pytest

import oracle
import vclgb_gen as gen
from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-13
TOL32 = 1e-5


@pytest.fixture(scope="module")
def V():
    import torch
    import vclgb
    torch.cuda.set_device(0)
    return vclgb


def _check(V, rp, ci, v, x, alpha=1.0, beta=0.0, y0=None, ncols=None):
    import torch
    A = V.compressed_matrix(rp, ci, v, len(rp) - 1, ncols)
    y = None if y0 is None else torch.tensor(y0, device="cuda")
    out = V.prod(A, x, alpha=alpha, y=y, beta=beta).cpu().numpy()
    ref = oracle.spmv(rp, ci, v, x, alpha, beta, y0)
    return rel_err(out, ref), A


def test_golden_alpha_beta(V, golden):
    d = golden("spmv_lognormal.npz")
    err, A = _check(V, d["rp"], d["ci"], d["v"], d["x"], float(d["alpha"]), float(d["beta"]),
                    d["y0"])
    assert err < TOL64
    assert A.info().num_bins > 1  # lognormal rows are binned


def test_golden_row_blocks(V, golden):
    d = golden("spmv_lognormal.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"])
    rb = A.row_blocks().cpu().numpy().view(np.uint32)
    assert np.array_equal(rb, d["row_blocks"])


def test_golden_float32(V, golden):
    d = golden("spmv_f32_lognormal.npz")
    A = V.compressed_matrix(d["rp"], d["ci"], d["v"].astype(np.float32))
    y = V.prod(A, d["x"].astype(np.float32)).cpu().numpy()
    assert rel_err(y, d["yf"]) < TOL32


@pytest.mark.parametrize("case", ["lap2d", "lap3d", "lognormal", "convdiff", "diffusion3d"])
def test_matrices(V, case):
    if case == "lap2d":
        rp, ci, v = gen.laplace2d(100, 77)
    elif case == "lap3d":
        rp, ci, v = gen.laplace3d(40)
    elif case == "lognormal":
        rp, ci, v = gen.lognormal_random(50000, seed=3)
    elif case == "convdiff":
        rp, ci, v = gen.convdiff2d(90, peclet=30)
    else:
        rp, ci, v, _ = gen.diffusion3d(24, corr=4.0)
    x = np.random.default_rng(1).uniform(-1, 1, len(rp) - 1)
    err, _ = _check(V, rp, ci, v, x)
    assert err < TOL64


def test_edge_rows(V):
    # empty rows, single entries, rows longer than 1024 (block-per-row bin)
    rng = np.random.default_rng(7)
    n = 5000
    lens = rng.integers(0, 4, n)
    lens[::97] = 0
    lens[10] = 3000
    lens[4000] = 1025
    lens[4999] = 2047
    rows, cols = [], []
    for r, L in enumerate(lens):
        c = np.sort(rng.choice(n, size=L, replace=False))
        cols.append(c)
    rp = np.zeros(n + 1, np.uint32)
    rp[1:] = np.cumsum(lens)
    ci = np.concatenate(cols).astype(np.uint32)
    v = rng.standard_normal(ci.size)
    x = rng.uniform(-1, 1, n)
    err, A = _check(V, rp, ci, v, x, 2.0, 0.5, rng.uniform(-1, 1, n))
    assert err < TOL64


def test_window_length_classes(V):
    # every row-length class of the row-window kernel, both sides of each
    # class limit, rows longer than 4096 (block per row), a partial last window
    rng = np.random.default_rng(11)
    n, m = 3001, 12000
    limits = [0, 1, 4, 5, 8, 9, 16, 17, 32, 33, 64, 65, 128, 129, 4096, 4097, 9000]
    lens = rng.integers(0, 40, n)
    lens[rng.choice(n, len(limits) * 3, replace=False)] = np.repeat(limits, 3)
    lens[-1] = 4097
    cols = [np.sort(rng.choice(m, size=L, replace=False)) for L in lens]
    rp = np.zeros(n + 1, np.uint32)
    rp[1:] = np.cumsum(lens)
    ci = np.concatenate(cols).astype(np.uint32)
    v = rng.standard_normal(ci.size)
    x = rng.uniform(-1, 1, m)
    err, A = _check(V, rp, ci, v, x, ncols=m)
    assert err < TOL64 and A.info().num_bins > 1
    err, _ = _check(V, rp, ci, v, x, -1.5, 0.25, rng.uniform(-1, 1, n), ncols=m)
    assert err < TOL64


def test_rectangular_and_tiny(V):
    rp = np.array([0, 2, 2, 3], np.uint32)
    ci = np.array([0, 6, 3], np.uint32)
    v = np.array([1.5, -2.0, 4.0])
    x = np.arange(7, dtype=np.float64)
    err, _ = _check(V, rp, ci, v, x, ncols=7)
    assert err < TOL64


def test_strided_kat(V):
    # tests/src/sparse.cpp:163-177 strided 5x4 product through start/stride
    import torch
    rows = [{0: 2.0, 2: -1.0}, {0: 3.0, 2: -5.0}, {1: 5.0, 2: -2.0}, {2: 1.0, 3: -6.0},
            {1: 7.0, 2: -5.0}]
    rp = np.zeros(6, np.uint32)
    ci, v = [], []
    for i, r in enumerate(rows):
        for c in sorted(r):
            ci.append(c)
            v.append(r[c])
        rp[i + 1] = len(ci)
    A = V.compressed_matrix(rp, np.array(ci, np.uint32), np.array(v), 5, 4)
    rhs = torch.arange(1, 12, dtype=torch.float64, device="cuda") * 0.5
    y = torch.full((16,), 7.0, dtype=torch.float64, device="cuda")
    V.prod(A, rhs, y=y, x_start=3, x_stride=2, y_start=1, y_stride=3)
    h = rhs.cpu().numpy()
    expect = np.full(16, 7.0)
    for i, r in enumerate(rows):
        expect[1 + 3 * i] = sum(val * h[3 + 2 * c] for c, val in r.items())
    assert np.array_equal(y.cpu().numpy(), expect)


def test_full_size_laplace3d_128(V):
    # full-size 128^3 7-point: compare against the oracle (OpenMP) end to end
    rp, ci, v = gen.laplace3d(128)
    x = np.random.default_rng(1).uniform(-1, 1, len(rp) - 1)
    err, A = _check(V, rp, ci, v, x)
    assert err < TOL64
    inf = A.info()
    assert inf.num_bins == 1 and inf.nnz == 14581760


def test_inner_prod_norm(V):
    import torch
    rng = np.random.default_rng(3)
    a = rng.standard_normal(1000003)
    b = rng.standard_normal(1000003)
    ta, tb = torch.tensor(a, device="cuda"), torch.tensor(b, device="cuda")
    assert abs(V.inner_prod(ta, tb).item() - np.dot(a, b)) < 1e-10 * abs(np.dot(a, b)) + 1e-9
    assert abs(V.norm_2(ta).item() - np.linalg.norm(a)) < 1e-12 * np.linalg.norm(a)
    # deterministic: repeated reductions give identical bits
    r1 = V.inner_prod(ta, tb).item()
    r2 = V.inner_prod(ta, tb).item()
    assert r1 == r2
