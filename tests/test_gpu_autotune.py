"""Per-matrix SpMV autotuner: the chosen form (CSR kernel, SELL-C-sigma with a
tuned slice height and sort window, HYB or ELL) gives the same product as the
CSR kernel within the FP64 SpMV tolerance, is no slower than it on the
tuner's own timing, and carries through the solvers (same iteration counts
and solutions within the solver tolerances)."""
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


@pytest.mark.parametrize("case", ["lognormal", "laplace3d", "lognormal_f32"])
def test_autotuned_product(V, case):
    import torch
    if case.startswith("lognormal"):
        rp, ci, v = gen.lognormal_random(200000, mu=2.5, sigma=1.0, hi=2000, seed=5)
    else:
        rp, ci, v = gen.laplace3d(64)
    dt = np.float32 if case.endswith("f32") else np.float64
    n = len(rp) - 1
    A = V.compressed_matrix(rp, ci, v.astype(dt))
    x = torch.tensor(np.random.default_rng(6).uniform(-1, 1, n).astype(dt), device="cuda")
    y_csr = V.prod(A, x).cpu().numpy()
    info = A.autotune()
    assert info["candidates"] >= 2
    assert info["us_best"] <= info["us_csr"]
    y = V.prod(A, x).cpu().numpy()
    tol = 1e-13 if dt == np.float64 else 1e-5
    assert rel_err(y, y_csr) < tol
    assert rel_err(y, oracle.spmv(rp, ci, v, x.cpu().numpy().astype(np.float64))) < tol
    A.autotune_clear()
    assert np.array_equal(V.prod(A, x).cpu().numpy(), y_csr)


def test_autotuned_form_in_solvers(V):
    import torch
    rp, ci, v = gen.lognormal_random(200000, mu=2.5, sigma=1.0, hi=2000, seed=7)
    n = len(rp) - 1
    b = torch.tensor(gen.rhs_uniform(n, 8), device="cuda")
    A = V.compressed_matrix(rp, ci, v)
    P = V.jacobi_precond(A)
    out = {}
    for tuned in (False, True):
        if tuned:
            A.autotune()
        tag = V.bicgstab_tag(1e-10, 3000)
        x = V.solve(A, b, tag, P).cpu().numpy()
        gtag = V.gmres_tag(1e-10, 3000, 30)
        xg = V.solve(A, b, gtag, P).cpu().numpy()
        out[tuned] = (x, tag.iters(), xg, gtag.iters())
    assert iters_close(out[True][1], out[False][1])
    assert rel_err(out[True][0], out[False][0]) < 1e-8
    assert iters_close(out[True][3], out[False][3])
    assert rel_err(out[True][2], out[False][2]) < 1e-8
