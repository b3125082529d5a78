"""Generates the golden fixtures in this directory by running ViennaCL's own
host/OpenMP backend (oracle/_ref/ref_driver, compiled from the reference
headers by oracle/Makefile) on small seeded inputs.  Each .npz stores the
inputs next to the reference outputs, so the tests need neither the reference
tree nor a particular numpy random stream.

Run from the repository root:  python tests/golden/make_golden.py
GMRES fixtures are produced with OMP_NUM_THREADS=1 (the host stage-1 kernel's
result depends on the thread count).
"""
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "viennacl-dev_gb300"))
import oracle  # noqa: E402
import vclgb_gen as gen  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def save(name, **arrays):
    np.savez_compressed(os.path.join(OUT, name), **arrays)
    print("wrote", name, sum(a.nbytes for a in map(np.asarray, arrays.values())))


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    assert oracle.have_ref(), "reference driver not built (needs the ViennaCL tree)"

    # SpMV with alpha/beta and the CSR-adaptive row blocks, lognormal rows incl. long ones
    rp, ci, v = gen.lognormal_random(3001, mu=2.5, sigma=1.0, hi=1500, seed=11)
    n = len(rp) - 1
    rng = np.random.default_rng(12)
    x = rng.uniform(-1, 1, n)
    y0 = rng.uniform(-1, 1, n)
    r = oracle.run_ref("spmv", rp, ci, v, args=(1.5, -0.5), x=x, y0=y0)
    save("spmv_lognormal.npz", rp=rp, ci=ci, v=v, x=x, y0=y0, alpha=1.5, beta=-0.5,
         y=r["y"], row_blocks=r["row_blocks"])
    r = oracle.run_ref("spmv_f32", rp, ci, v, x=x)
    save("spmv_f32_lognormal.npz", rp=rp, ci=ci, v=v, x=x, yf=r["yf"])

    # format conversions + per-format SpMV (n % 32 != 0 so the host SELL SpMV is valid)
    rp, ci, v = gen.lognormal_random(1999, mu=2.0, sigma=0.8, hi=60, seed=13)
    n = len(rp) - 1
    x = np.random.default_rng(14).uniform(-1, 1, n)
    r = oracle.run_ref("formats", rp, ci, v, args=(32, 0.8), x=x)
    save("formats_lognormal.npz", rp=rp, ci=ci, v=v, x=x, C=32, threshold=0.8,
         **{k: r[k] for k in r if k.startswith(("ell", "sell", "hyb", "y_"))})
    # HYB with an empty tail (uniform rows) -> placeholder entry
    rp, ci, v = gen.laplace2d(20, 17)
    n = len(rp) - 1
    x = np.random.default_rng(15).uniform(-1, 1, n)
    r = oracle.run_ref("formats", rp, ci, v, args=(32, 0.8), x=x)
    save("formats_laplace2d.npz", rp=rp, ci=ci, v=v, x=x, C=32, threshold=0.8,
         **{k: r[k] for k in r if k.startswith(("ell", "sell", "hyb", "y_"))})
    r = oracle.run_ref("hyb_f32_width", rp, ci, v, args=(0.8,))
    save("hyb_f32_laplace2d.npz", rp=rp, ci=ci, v=v, width=r["hybf_width"])

    # CG: pipelined (no preconditioner), Jacobi, ILU0 on the 2D Laplacian
    rp, ci, v = gen.laplace2d(40, 40)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 0)
    res = {}
    for pc in ("none", "jacobi", "ilu0"):
        r = oracle.run_ref("cg", rp, ci, v, args=(1e-8, 2000, pc), b=b)
        res["x_" + pc] = r["x"]
        res["iters_" + pc] = r["iters"]
        res["error_" + pc] = r["error"]
    save("cg_laplace2d.npz", rp=rp, ci=ci, v=v, b=b, tol=1e-8, max_iters=2000, **res)

    # BiCGStab (pipelined / Jacobi) and GMRES(30) on convection-diffusion
    rp, ci, v = gen.convdiff2d(30, 28, peclet=20.0, shift=0.05)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 3)
    res = {}
    for pc in ("none", "jacobi"):
        r = oracle.run_ref("bicgstab", rp, ci, v, args=(1e-10, 400, pc), b=b)
        res["x_" + pc] = r["x"]
        res["iters_" + pc] = r["iters"]
        res["error_" + pc] = r["error"]
    save("bicgstab_convdiff.npz", rp=rp, ci=ci, v=v, b=b, tol=1e-10, max_iters=400, **res)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    out = subprocess.run([sys.executable, "-c", (
        "import sys; sys.path.insert(0, %r); import oracle, numpy as np; "
        "d = np.load(%r); r = oracle.run_ref('gmres', d['rp'], d['ci'], d['v'], "
        "args=(1e-10, 600, 'none', 30), b=d['b']); "
        "np.savez_compressed(%r, rp=d['rp'], ci=d['ci'], v=d['v'], b=d['b'], tol=1e-10, "
        "max_iters=600, krylov_dim=30, x=r['x'], iters=r['iters'], error=r['error'])")
        % (os.path.join(ROOT, "oracle"), os.path.join(OUT, "bicgstab_convdiff.npz"),
           os.path.join(OUT, "gmres_convdiff_1thread.npz"))], env=env, check=True)
    print("wrote gmres_convdiff_1thread.npz", out.returncode)

    # mixed_precision_cg
    rp, ci, v = gen.laplace2d(36, 36)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 5)
    r = oracle.run_ref("mixed_cg", rp, ci, v, args=(1e-8, 3000, "none", 1e-2), b=b)
    save("mixed_cg_laplace2d.npz", rp=rp, ci=ci, v=v, b=b, tol=1e-8, max_iters=3000,
         inner_tol=1e-2, x=r["x"], iters=r["iters"], error=r["error"])

    # adjoint: forward solve and the transpose solve A^T lambda = x - x_t with the
    # reference host backend (Jacobi-BiCGStab for the nonsymmetric case -- the
    # host GMRES stagnates below 1e-12 on it because of its stage-1 defect --
    # and Jacobi-PCG for the SPD diffusion case); dL/dA = -lambda_i x_j
    rp, ci, v = gen.convdiff2d(20, 18, peclet=10.0, shift=0.1)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 21)
    xt = np.random.default_rng(22).uniform(0.0, 1.0, n)
    x = oracle.run_ref("bicgstab", rp, ci, v, args=(1e-14, 3000, "jacobi"), b=b)["x"]
    trp, tci, tv, mp = oracle.transpose(n, n, rp, ci, v)
    lam = oracle.run_ref("bicgstab", trp, tci, tv, args=(1e-14, 3000, "jacobi"), b=x - xt)["x"]
    rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    save("adjoint_convdiff.npz", rp=rp, ci=ci, v=v, b=b, xt=xt, x=x, lam=lam,
         dLdA=-lam[rows] * x[ci], trp=trp, tci=tci, tv=tv, map=mp)
    rp, ci, v, _ = gen.diffusion2d_edges(24, contrast=1e3, seed=4)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 23)
    xt = np.random.default_rng(24).uniform(0.0, 1.0, n)
    x = oracle.run_ref("cg", rp, ci, v, args=(1e-13, 5000, "jacobi"), b=b)["x"]
    lam = oracle.run_ref("cg", rp, ci, v, args=(1e-13, 5000, "jacobi"), b=x - xt)["x"]
    rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    save("adjoint_diffusion2d.npz", rp=rp, ci=ci, v=v, b=b, xt=xt, x=x, lam=lam,
         dLdA=-lam[rows] * x[ci])

    # ILU0 factors, level sets (L and U) and the level-scheduled apply
    rp, ci, v = gen.convdiff2d(23, 19, peclet=5.0, shift=0.2)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 7)
    r = oracle.run_ref("ilu0", rp, ci, v, b=b)
    save("ilu0_convdiff.npz", rp=rp, ci=ci, v=v, b=b,
         **{k: r[k] for k in r if k.startswith(("L_", "U_")) or k in ("lu", "udiag", "z")})


if __name__ == "__main__":
    main()
