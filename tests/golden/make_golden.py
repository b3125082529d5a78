"""Generates the golden fixtures in this directory by running ViennaCL's own
host/OpenMP backend (oracle/_ref/ref_driver, compiled from the reference
headers by oracle/Makefile) on small seeded inputs.  Each .npz stores the
inputs next to the reference outputs, so the tests need neither the reference
tree nor a particular numpy random stream.

Run from the repository root:  python tests/golden/make_golden.py
(python tests/golden/make_golden.py coo | row_scaling | matrix_market | cuthill_mckee |
 chow_patel | block_ilu | gmres_precond | trisolve writes only
that fixture; matrix_market also writes the input files under tests/golden/mm/)
GMRES fixtures are produced with OMP_NUM_THREADS=1 (the host stage-1 kernel's
result depends on the thread count).
"""
import os
import subprocess
import sys
import tempfile

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
    gmres_precond_fixture()
    trisolve_fixture()

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

    coo_fixture()
    row_scaling_fixture()
    mm_fixture()
    cm_fixture()
    chow_patel_fixture()
    block_ilu_fixture()


def coo_fixture():
    """coordinate_matrix: the reference's arrays, its 65 group boundaries and
    its host product; two leading empty rows exercise the group rule."""
    rp, ci, v = gen.lognormal_random(1500, mu=2.0, sigma=0.9, hi=200, seed=21)
    ncols = len(rp) - 1
    rp = np.concatenate([[0, 0], rp]).astype(np.uint32)
    n = len(rp) - 1
    rng = np.random.default_rng(25)
    x = rng.uniform(-1, 1, ncols)
    y0 = rng.uniform(-1, 1, n)
    r = oracle.run_ref("coo", rp, ci, v, ncols=ncols, args=(1.5, -0.5), x=x, y0=y0)
    save("coo_lognormal.npz", rp=rp, ci=ci, v=v, ncols=ncols, x=x, y0=y0, alpha=1.5, beta=-0.5,
         nnz=r["coo_nnz"], coords=r["coo_coords"], elems=r["coo_elems"],
         groups=r["coo_groups"], y=r["y_coo"])



def row_scaling_fixture():
    """row_scaling: the three row-norm diagonals (row_info) and BiCGStab / CG
    solves preconditioned by them."""
    rp, ci, v = gen.convdiff2d(30, 28, peclet=20.0, shift=0.05)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 3)
    r = oracle.run_ref("row_norms", rp, ci, v)
    res = {"norm%d" % p: r["norm%d" % p] for p in range(3)}
    for p in range(3):
        s = oracle.run_ref("bicgstab", rp, ci, v, args=(1e-10, 2000, "row%d" % p), b=b)
        res["x_bicgstab_row%d" % p] = s["x"]
        res["iters_bicgstab_row%d" % p] = s["iters"]
        res["error_bicgstab_row%d" % p] = s["error"]
    lp, lc, lv = gen.laplace2d(40, 40)
    lb = gen.rhs_uniform(len(lp) - 1, 0)
    s = oracle.run_ref("cg", lp, lc, lv, args=(1e-8, 2000, "row2"), b=lb)
    save("row_scaling_convdiff.npz", rp=rp, ci=ci, v=v, b=b, lp=lp, lc=lc, lv=lv, lb=lb,
         x_cg_row2=s["x"], iters_cg_row2=s["iters"], error_cg_row2=s["error"], **res)



MM_DIR = os.path.join(OUT, "mm")


def _mm_write(name, header, size, entries, comments=(), blank=False, fmt="%d %d %s"):
    lines = [header] + list(comments) + [size]
    for i, e in enumerate(entries):
        lines.append(fmt % e if isinstance(e, tuple) else e)
        if blank and i % 7 == 3:
            lines.append("")
    with open(os.path.join(MM_DIR, name), "w") as f:
        f.write("\n".join(lines) + "\n")


def mm_inputs():
    """Small synthetic MatrixMarket files (seeded) covering the reader's rules:
    general / symmetric / pattern / complex, comments, blank lines, mixed-case
    header words, leading and trailing spaces, duplicate positions (the later
    one wins), 0-based indices, lines after the announced entries, and the
    error cases (bad header words, array format, index out of range, too few
    entries, a missing value)."""
    os.makedirs(MM_DIR, exist_ok=True)
    rng = np.random.default_rng(31)

    def rand_entries(n, m, k, sym=False):
        out = []
        for _ in range(k):
            i, j = int(rng.integers(1, n + 1)), int(rng.integers(1, m + 1))
            if sym and j > i:
                i, j = j, i
            out.append((i, j, repr(float(rng.normal()))))
        return out

    g = rand_entries(40, 30, 150)
    g += [(g[5][0], g[5][1], "7.25"), (g[9][0], g[9][1], "-0.5")]  # duplicates: later wins
    _mm_write("general.mtx", "%%MatrixMarket matrix coordinate real general", "40 30 %d" % len(g),
              g, comments=("% a comment", "%another one"), blank=True)
    _mm_write("general_case.mtx", "%%MATRIXMARKET Matrix Coordinate REAL General",
              "   12 12 20  ", ["  %d %d %s  " % e for e in rand_entries(12, 12, 20)])
    s = rand_entries(50, 50, 120, sym=True) + [(3, 3, "4.0"), (7, 2, "1.5"), (2, 7, "2.5")]
    _mm_write("symmetric.mtx", "%%MatrixMarket matrix coordinate real symmetric",
              "50 50 %d" % len(s), s)
    p = [(i, j) for i, j, _ in rand_entries(25, 35, 60)]
    _mm_write("pattern.mtx", "%%MatrixMarket matrix coordinate pattern general", "25 35 60", p,
              fmt="%d %d")
    c = [(i, j, "%s %s" % (v, repr(float(rng.normal())))) for i, j, v in rand_entries(20, 20, 45)]
    _mm_write("complex.mtx", "%%MatrixMarket matrix coordinate complex general", "20 20 45", c)
    z = [(i - 1, j - 1, v) for i, j, v in rand_entries(15, 15, 30)]
    _mm_write("zero_based.mtx", "%%MatrixMarket matrix coordinate real general", "15 15 30", z)
    e = rand_entries(10, 10, 12)
    _mm_write("extra_lines.mtx", "%%MatrixMarket matrix coordinate real general", "10 10 8",
              e, comments=("%",))
    _mm_write("bad_word.mtx", "%%MatrixMarket tensor coordinate real general", "5 5 2",
              [(1, 1, "1.0"), (2, 2, "2.0")])
    _mm_write("bad_field.mtx", "%%MatrixMarket matrix coordinate integer general", "5 5 2",
              [(1, 1, "1"), (2, 2, "2")])
    _mm_write("bad_symmetry.mtx", "%%MatrixMarket matrix coordinate real skew-symmetric", "5 5 2",
              [(2, 1, "1.0"), (3, 2, "2.0")])
    _mm_write("array.mtx", "%%MatrixMarket matrix array real general", "2 2",
              ["1.0", "2.0", "3.0", "4.0"])
    _mm_write("out_of_range.mtx", "%%MatrixMarket matrix coordinate real general", "5 5 3",
              [(1, 1, "1.0"), (6, 2, "2.0"), (3, 3, "3.0")])
    _mm_write("too_few.mtx", "%%MatrixMarket matrix coordinate real general", "5 5 4",
              [(1, 1, "1.0"), (2, 2, "2.0")])
    _mm_write("missing_value.mtx", "%%MatrixMarket matrix coordinate real general", "5 5 2",
              [(1, 1, "1.0"), "2 2"])


MM_CASES = [("general.mtx", 1), ("general_case.mtx", 1), ("symmetric.mtx", 1),
            ("pattern.mtx", 1), ("complex.mtx", 1), ("zero_based.mtx", 0), ("extra_lines.mtx", 1),
            ("bad_word.mtx", 1), ("bad_field.mtx", 1), ("bad_symmetry.mtx", 1), ("array.mtx", 1),
            ("out_of_range.mtx", 1), ("too_few.mtx", 1), ("missing_value.mtx", 1)]


def mm_fixture():
    """The reference reader's result for each file: its return value (0 =
    error) and the matrix as CSR (rows sorted by column, as std::map holds them)."""
    mm_inputs()
    res = {}
    for name, base in MM_CASES:
        with tempfile.TemporaryDirectory() as d:
            subprocess.run([oracle.REF_DRIVER, "mm_read", d, os.path.join(MM_DIR, name),
                            str(base)], check=True, stdout=subprocess.DEVNULL,
                           stderr=subprocess.DEVNULL)
            key = name[:-4]
            for f in ("ret", "rp", "ci"):
                res[key + "__" + f] = np.fromfile(os.path.join(d, "mm_%s.u32" % f), np.uint32)
            res[key + "__v"] = np.fromfile(os.path.join(d, "mm_v.f64"), np.float64)
    save("matrix_market.npz", **res)



def _sym_permute(rp, ci, v, p):
    """B(p[i], p[j]) = A(i, j) as CSR with ascending columns (numpy)."""
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    r2, c2 = p[rows], p[ci.astype(np.int64)]
    order = np.lexsort((c2, r2))
    rp2 = np.zeros(n + 1, np.int64)
    np.add.at(rp2, r2 + 1, 1)
    return np.cumsum(rp2).astype(np.uint32), c2[order].astype(np.uint32), v[order]


def cm_fixture():
    """Cuthill-McKee: a 2D Laplacian with scrambled numbering (two copies, so
    there are two components) plus isolated nodes, and a convection-diffusion
    matrix; permutations from both tags and the bandwidths before and after."""
    rng = np.random.default_rng(41)
    rp, ci, v = gen.laplace2d(24, 18)
    n1 = len(rp) - 1
    # block diagonal: Laplacian, Laplacian, 5 diagonal-only rows
    blocks = [(rp, ci, v, 0), (rp, ci, v, n1)]
    rows_r, rows_c, rows_v = [], [], []
    for brp, bci, bv, off in blocks:
        r = np.repeat(np.arange(n1), np.diff(brp.astype(np.int64))) + off
        rows_r.append(r)
        rows_c.append(bci.astype(np.int64) + off)
        rows_v.append(bv)
    iso = np.arange(2 * n1, 2 * n1 + 5)
    rows_r.append(iso)
    rows_c.append(iso)
    rows_v.append(np.full(5, 2.0))
    r, c, vv = np.concatenate(rows_r), np.concatenate(rows_c), np.concatenate(rows_v)
    n = 2 * n1 + 5
    order = np.lexsort((c, r))
    brp = np.zeros(n + 1, np.int64)
    np.add.at(brp, r + 1, 1)
    brp = np.cumsum(brp).astype(np.uint32)
    bci, bv = c[order].astype(np.uint32), vv[order]
    rp, ci, v = _sym_permute(brp, bci, bv, rng.permutation(n))
    res = {}
    for key, args in (("cm", (0, 0, 0)), ("acm_a0_g1", (1, 0.0, 1)), ("acm_a05_g2", (1, 0.5, 2))):
        out = oracle.run_ref("cm", rp, ci, v, args=args)
        res["perm_" + key], res["bw_" + key] = out["perm"], out["bw"]
    cp, cc, cv = gen.convdiff2d(17, 23, peclet=5.0, shift=0.2)
    cp, cc, cv = _sym_permute(cp, cc, cv, np.random.default_rng(42).permutation(len(cp) - 1))
    out = oracle.run_ref("cm", cp, cc, cv, args=(0, 0, 0))
    save("cuthill_mckee.npz", rp=rp, ci=ci, v=v, cp=cp, cc=cc, cv=cv, perm_cd=out["perm"],
         bw_cd=out["bw"], **res)


def chow_patel_fixture():
    """Chow-Patel ILU on a convection-diffusion matrix and Chow-Patel ICC on a
    variable-coefficient diffusion matrix: the Neumann matrices and diagonals
    of detail::precondition for two tags, the applies, and BiCGStab / CG
    solves preconditioned by them (default tag)."""
    cp, cc, cv = gen.convdiff2d(23, 19, peclet=10.0, shift=0.05)
    sp, sc, sv, _ = gen.diffusion2d_edges(21, contrast=1e2, seed=43)
    res = {}
    for name, (rp, ci, v) in (("cd", (cp, cc, cv)), ("sd", (sp, sc, sv))):
        n = len(rp) - 1
        b = gen.rhs_uniform(n, 44)
        res["b_" + name] = b
        for sweeps, iters in ((3, 2), (1, 4)):
            out = oracle.run_ref("chow_patel", rp, ci, v, args=(sweeps, iters), b=b)
            tag = "%s_%d_%d_" % (name, sweeps, iters)
            for k in ("cpl_rp", "cpl_ci", "cpl_v", "cpl_diag", "cpu_rp", "cpu_ci", "cpu_v",
                      "cpu_diag", "cp_ilu_z", "icl_rp", "icl_ci", "icl_v", "icl_diag", "iclt_rp",
                      "iclt_ci", "iclt_v", "cp_icc_z"):
                res[tag + k] = out[k]
    s = oracle.run_ref("bicgstab", cp, cc, cv, args=(1e-10, 2000, "cpilu"), b=res["b_cd"])
    res.update(x_bicgstab_cpilu=s["x"], iters_bicgstab_cpilu=s["iters"],
               error_bicgstab_cpilu=s["error"])
    s = oracle.run_ref("cg", sp, sc, sv, args=(1e-10, 2000, "cpicc"), b=res["b_sd"])
    res.update(x_cg_cpicc=s["x"], iters_cg_cpicc=s["iters"], error_cg_cpicc=s["error"])
    save("chow_patel.npz", cp=cp, cc=cc, cv=cv, sp=sp, sc=sc, sv=sv, **res)


def block_ilu_fixture():
    """block_ilu_precond<compressed_matrix, ilu0_tag> with 1, 8 and 37 blocks
    (the default split, n not divisible by the count) on a convection-diffusion
    matrix: the blocks' ILU0 factors side by side and the apply; BiCGStab
    preconditioned by it (8 blocks)."""
    rp, ci, v = gen.convdiff2d(29, 23, peclet=10.0, shift=0.02)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 47)
    res = {}
    for nb in (1, 8, 37):
        out = oracle.run_ref("block_ilu", rp, ci, v, args=(nb,), b=b)
        res["lu_%d" % nb], res["z_%d" % nb] = out["bilu_lu"], out["bilu_z"]
    s = oracle.run_ref("bicgstab", rp, ci, v, args=(1e-10, 2000, "bilu8"), b=b)
    save("block_ilu.npz", rp=rp, ci=ci, v=v, b=b, x_bicgstab_bilu8=s["x"],
         iters_bicgstab_bilu8=s["iters"], error_bicgstab_bilu8=s["error"], **res)


def gmres_precond_fixture():
    """Preconditioned GMRES (the reference's Householder variant, gmres.hpp:449-631)
    with Jacobi, ILU0, row scaling and Chow-Patel ILU, Krylov dimensions 30 and 10,
    on a convection-diffusion matrix; one host thread (bit-reproducible sums)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    assert oracle.have_ref(), "reference driver not built (needs the ViennaCL tree)"
    rp, ci, v = gen.convdiff2d(48, 44, peclet=25.0, shift=0.02)
    n = len(rp) - 1
    b = gen.rhs_uniform(n, 6)
    np.savez(os.path.join(tempfile.gettempdir(), "gmres_precond_in.npz"), rp=rp, ci=ci, v=v, b=b)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([sys.executable, "-c", (
        "import sys; sys.path.insert(0, %r); import oracle, numpy as np; "
        "d = np.load(%r); res = {}\n"
        "for pc in ('jacobi', 'ilu0', 'row1', 'cpilu'):\n"
        "    for kd in (30, 10):\n"
        "        r = oracle.run_ref('gmres', d['rp'], d['ci'], d['v'], args=(1e-10, 1000, pc, kd), b=d['b'])\n"
        "        key = '%%s_%%d' %% (pc, kd)\n"
        "        res['x_' + key] = r['x']; res['iters_' + key] = r['iters']; res['error_' + key] = r['error']\n"
        "np.savez_compressed(%r, rp=d['rp'], ci=d['ci'], v=d['v'], b=d['b'], tol=1e-10, "
        "max_iters=1000, **res)")
        % (os.path.join(ROOT, "oracle"), os.path.join(tempfile.gettempdir(), "gmres_precond_in.npz"),
           os.path.join(OUT, "gmres_precond_convdiff.npz"))], env=env, check=True)
    print("wrote gmres_precond_convdiff.npz")


def trisolve_matrices():
    """The 5x5 literal matrix of the reference's resize test (tests/src/sparse.cpp:
    221-225), a row-scaled convection-diffusion matrix (unit diagonal, so the
    unit-triangular solves stay bounded) and a lognormal random matrix."""
    lit = np.array([[10.0, 0.1, 0.2, 0.3, 0.4], [1.0, 1.1, 1.2, 1.3, 1.4],
                    [2.0, 2.1, 2.2, 2.3, 2.4], [3.0, 3.1, 3.2, 3.3, 3.4],
                    [4.0, 4.1, 4.2, 4.3, 4.4]])
    out = {"literal5": (np.arange(0, 26, 5, dtype=np.uint32),
                        np.tile(np.arange(5, dtype=np.uint32), 5), lit.ravel())}
    rp, ci, v = gen.convdiff2d(30, 28, peclet=20.0, shift=0.05)
    d = oracle.diag(rp, ci, v)
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp.astype(np.int64)))
    out["convdiff_scaled"] = (rp, ci, v / d[rows])
    out["lognormal"] = gen.lognormal_random(2000, mu=2.0, sigma=0.8, hi=60, seed=21)
    return out


def trisolve_fixture():
    """inplace_solve(A, b, tag) and inplace_solve(trans(A), b, tag) for the four
    tags (host_based/sparse_matrix_operations.hpp:537-1090), b = 1 + U[0, 1)
    as the reference's test builds its right-hand side (sparse.cpp:346)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    assert oracle.have_ref(), "reference driver not built (needs the ViennaCL tree)"
    res = {}
    for name, (rp, ci, v) in trisolve_matrices().items():
        b = 1.0 + np.random.default_rng(22).uniform(0, 1, len(rp) - 1)
        r = oracle.run_ref("trisolve", rp, ci, v, b=b)
        res.update({name + "_rp": rp, name + "_ci": ci, name + "_v": v, name + "_b": b})
        for k in r:
            if k.startswith("tri_"):
                res[name + "_" + k] = r[k]
    save("trisolve.npz", **res)


if __name__ == "__main__":
    if sys.argv[1:] == ["trisolve"]:
        trisolve_fixture()
    elif sys.argv[1:] == ["gmres_precond"]:
        gmres_precond_fixture()
    elif sys.argv[1:] == ["coo"]:
        coo_fixture()
    elif sys.argv[1:] == ["row_scaling"]:
        row_scaling_fixture()
    elif sys.argv[1:] == ["chow_patel"]:
        chow_patel_fixture()
    elif sys.argv[1:] == ["block_ilu"]:
        block_ilu_fixture()
    elif sys.argv[1:] == ["matrix_market"]:
        mm_fixture()
    elif sys.argv[1:] == ["cuthill_mckee"]:
        cm_fixture()
    else:
        main()
