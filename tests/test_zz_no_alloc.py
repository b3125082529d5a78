"""vclgbHybSpmvNoAlloc: the HYB product that allocates nothing, for callers
that may not allocate device memory when they call in (a plug-in whose host
application owns all device allocations, a service with a fixed memory budget,
a latency-bound loop).  It is checked through the C ABI against the regular
HYB product (vclgbSpmv) on two calls in a row, within the FP64 SpMV tolerance
of the other tests.  The file is collected last; it passes on its own and
after the rest of the suite."""
import ctypes

import numpy as np
import pytest

import oracle
import vclgb_gen as gen
from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _u32(t):
    return t.cpu().numpy().view(np.uint32)


def test_no_alloc_hyb_matches_regular_entry_point():
    import torch
    import vclgb as V
    torch.cuda.set_device(0)
    lib = V.load_library()
    # lognormal rows: long rows spill into the tail across many warp chunks
    rp, ci, v = gen.lognormal_random(40000, mu=2.5, sigma=1.2, hi=2000, seed=19)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v)
    H = V.hyb_matrix(A, 0.8)
    inf = H.info()
    w = inf.ell_width
    tail_nnz = int(_u32(H.export(2, n + 1, torch.int32))[-1])
    assert 0 < tail_nnz <= (1 << 23)
    ell_coords = H.export(0, n * w, torch.int32)
    ell_elems = H.export(1, n * w, torch.float64)
    tail_rp = H.export(2, n + 1, torch.int32)
    tail_ci = H.export(3, inf.tail_nnz, torch.int32)
    tail_v = H.export(4, inf.tail_nnz, torch.float64)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(23)
    y_prev = None
    for call, (alpha, beta) in enumerate(((1.0, 0.0), (-0.5, 2.0))):
        x = torch.tensor(rng.uniform(-1, 1, n), device="cuda")
        y0 = rng.uniform(-1, 1, n)
        y_new = torch.tensor(y0, device="cuda")
        y_ref = torch.tensor(y0, device="cuda")
        st = lib.vclgbHybSpmvNoAlloc(ctypes.c_void_p(stream), V.FLOAT64, n, w,
                                     ctypes.c_void_p(ell_coords.data_ptr()),
                                     ctypes.c_void_p(ell_elems.data_ptr()),
                                     ctypes.c_void_p(tail_rp.data_ptr()),
                                     ctypes.c_void_p(tail_ci.data_ptr()),
                                     ctypes.c_void_p(tail_v.data_ptr()), tail_nnz, alpha,
                                     ctypes.c_void_p(x.data_ptr()), beta,
                                     ctypes.c_void_p(y_new.data_ptr()))
        assert st == V.SUCCESS
        V.prod(H, x, alpha=alpha, y=y_ref, beta=beta)  # the existing entry point
        torch.cuda.synchronize()
        got, want = y_new.cpu().numpy(), y_ref.cpu().numpy()
        assert rel_err(got, want) < TOL, call
        assert rel_err(got, oracle.spmv(rp, ci, v, x.cpu().numpy(), alpha, beta, y0)) < TOL
        if y_prev is not None:
            assert not np.array_equal(got, y_prev)  # the second call computed anew
        y_prev = got


def test_no_alloc_rejects_a_tail_beyond_its_scratch():
    import vclgb as V
    lib = V.load_library()
    st = lib.vclgbHybSpmvNoAlloc(None, V.FLOAT64, 10, 1, None, None, None, None, None,
                                 (1 << 23) + 1, 1.0, None, 0.0, None)
    assert st == V.INVALID_ARGUMENT


def _call(lib, V, prec, n, w, ell_coords, ell_elems, trp, tci, tv, tnnz, alpha, x, beta, y):
    import torch
    p = lambda t: ctypes.c_void_p(t.data_ptr() if t is not None and t.numel() else 0)
    stream = torch.cuda.current_stream().cuda_stream
    return lib.vclgbHybSpmvNoAlloc(ctypes.c_void_p(stream), prec, n, w, p(ell_coords),
                                   p(ell_elems), p(trp), p(tci), p(tv), tnnz, alpha, p(x), beta,
                                   p(y))


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("case", ["hyb_lognormal", "ell_only_narrow", "ell_only_wide",
                                  "tail_only"])
def test_no_alloc_precisions_and_parts(dtype, case):
    # both precisions; a lognormal HYB with both parts; an empty tail with an
    # ELL width among the specialised kernels' (the HYB of a 2D Laplacian,
    # width 5, the placeholder tail entry) and with a width beyond them (a
    # lognormal matrix at threshold 1.0: every row in the ELL part); an empty
    # ELL part (width 0, the whole matrix as the CSR tail).  Two calls each,
    # against the regular entry point (vclgbSpmv) and the oracle
    import torch
    import vclgb as V
    torch.cuda.set_device(0)
    lib = V.load_library()
    tdt = torch.float64 if dtype == "f64" else torch.float32
    prec = V.FLOAT64 if dtype == "f64" else V.FLOAT32
    tol = TOL if dtype == "f64" else 1e-5
    if case in ("hyb_lognormal", "tail_only"):
        rp, ci, v = gen.lognormal_random(20000, mu=2.0, sigma=1.0, hi=600, seed=29)
    elif case == "ell_only_wide":
        rp, ci, v = gen.lognormal_random(20000, mu=2.0, sigma=0.6, hi=40, seed=31)
    else:
        rp, ci, v = gen.laplace2d(97, 83)
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v.astype(np.float64 if dtype == "f64" else np.float32))
    if case == "tail_only":
        w, tnnz = 0, int(rp[-1])
        ell_coords = ell_elems = None
        trp = torch.tensor(rp.view(np.int32), device="cuda")
        tci = torch.tensor(ci.view(np.int32), device="cuda")
        tv = torch.tensor(v, dtype=tdt, device="cuda")
    else:
        H = V.hyb_matrix(A, 1.0 if case == "ell_only_wide" else 0.8)
        inf = H.info()
        w = inf.ell_width
        trp = H.export(2, n + 1, torch.int32)
        tnnz = int(_u32(trp)[-1])
        ell_coords = H.export(0, n * w, torch.int32)
        ell_elems = H.export(1, n * w, tdt)
        tci = H.export(3, inf.tail_nnz, torch.int32)
        tv = H.export(4, inf.tail_nnz, tdt)
        if case == "ell_only_narrow":
            assert tnnz == 0 and w == 5
        elif case == "ell_only_wide":
            assert tnnz == 0 and w > 8
        else:
            assert tnnz > 0 and w > 0
    rng = np.random.default_rng(41)
    prev = None
    for alpha, beta in ((1.0, 0.0), (0.75, -1.5)):
        x = torch.tensor(rng.uniform(-1, 1, n), dtype=tdt, device="cuda")
        y0 = rng.uniform(-1, 1, n)
        y_new = torch.tensor(y0, dtype=tdt, device="cuda")
        y_ref = torch.tensor(y0, dtype=tdt, device="cuda")
        st = _call(lib, V, prec, n, w, ell_coords, ell_elems, trp, tci, tv, tnnz, alpha, x, beta,
                   y_new)
        assert st == V.SUCCESS
        V.prod(A, x, alpha=alpha, y=y_ref, beta=beta)  # the regular entry point
        torch.cuda.synchronize()
        got = y_new.cpu().numpy().astype(np.float64)
        assert rel_err(got, y_ref.cpu().numpy()) < tol
        want = oracle.spmv(rp, ci, v, x.cpu().numpy().astype(np.float64), alpha, beta,
                           y_new.new_tensor(y0).cpu().numpy().astype(np.float64))
        assert rel_err(got, want) < tol
        if prev is not None:
            assert not np.array_equal(got, prev)
        prev = got
