"""The CPU oracle (oracle/vcl_oracle.c) against ViennaCL's own host backend:
golden fixtures produced by tests/golden/make_golden.py, the small literal
matrices of the reference's tests/src/sparse.cpp, and -- where the reference
tree exists -- live runs of oracle/_ref/ref_driver."""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
import vclgb_gen as gen
from conftest import rel_err


def test_kat_strided_spmv():
    # tests/src/sparse.cpp:163-177: project(result, slice(1,3,5)) =
    #   prod(A, project(rhs, slice(3,2,4))) with the 5x4 literal matrix
    rows = [{0: 2.0, 2: -1.0}, {0: 3.0, 2: -5.0}, {1: 5.0, 2: -2.0}, {2: 1.0, 3: -6.0},
            {1: 7.0, 2: -5.0}]
    rp = np.zeros(6, np.uint32)
    ci, v = [], []
    for i, r in enumerate(rows):
        for c in sorted(r):
            ci.append(c)
            v.append(r[c])
        rp[i + 1] = len(ci)
    rhs = np.arange(1, 12, dtype=np.float64) * 0.5
    y = np.full(16, 7.0)
    out = oracle.spmv_strided(rp, np.array(ci, np.uint32), np.array(v), rhs, 3, 2, 1.0, 0.0,
                              y, 1, 3)
    expect = y.copy()
    for i, r in enumerate(rows):
        expect[1 + 3 * i] = sum(val * rhs[3 + 2 * c] for c, val in r.items())
    assert np.array_equal(out, expect)


def test_spmv_alpha_beta_golden(golden):
    d = golden("spmv_lognormal.npz")
    y = oracle.spmv(d["rp"], d["ci"], d["v"], d["x"], float(d["alpha"]), float(d["beta"]), d["y0"])
    assert rel_err(y, d["y"]) < 1e-14
    assert np.array_equal(oracle.row_blocks(d["rp"]), d["row_blocks"])


def test_coo_golden(golden):
    # coordinate_matrix copy (coordinate_matrix.hpp:46-101) incl. its group
    # boundaries, and the host COO product: both bit-exact
    d = golden("coo_lognormal.npz")
    C = oracle.coo(d["rp"], d["ci"], d["v"])
    assert C["nnz"] == int(d["nnz"][0]) and C["stored"] == int(d["nnz"][1])
    assert np.array_equal(C["coords"], d["coords"]) and np.array_equal(C["elems"], d["elems"])
    assert np.array_equal(C["groups"], d["groups"])
    assert d["groups"][1] == d["rp"][3] and d["groups"][63] == d["groups"][1]  # group rule
    n = len(d["rp"]) - 1
    y = oracle.coo_spmv(n, C, d["x"], float(d["alpha"]), float(d["beta"]), d["y0"])
    assert np.array_equal(y, d["y"])


def test_row_scaling_golden(golden):
    # row_info row norms (bit-exact) and the solves they precondition
    # (single thread: iteration count, estimate and solution identical)
    d = golden("row_scaling_convdiff.npz")
    for p in range(3):
        assert np.array_equal(oracle.row_norms(d["rp"], d["v"], p), d["norm%d" % p])
    oracle.set_threads(1)
    try:
        for p in range(3):
            x, it, err = oracle.solve("bicgstab", d["rp"], d["ci"], d["v"], d["b"], 1e-10, 2000,
                                      "row%d" % p)
            assert it == int(d["iters_bicgstab_row%d" % p]) and err == float(d["error_bicgstab_row%d" % p])
            assert rel_err(x, d["x_bicgstab_row%d" % p]) < 1e-12
        x, it, err = oracle.solve("cg", d["lp"], d["lc"], d["lv"], d["lb"], 1e-8, 2000, "row2")
        assert it == int(d["iters_cg_row2"]) and rel_err(x, d["x_cg_row2"]) < 1e-12
    finally:
        oracle.set_threads(oracle.max_threads())


CP_ILU_KEYS = (("l_rp", "cpl_rp"), ("l_ci", "cpl_ci"), ("l_v", "cpl_v"), ("diag_l", "cpl_diag"),
               ("u_rp", "cpu_rp"), ("u_ci", "cpu_ci"), ("u_v", "cpu_v"), ("diag_u", "cpu_diag"))
CP_ICC_KEYS = (("l_rp", "icl_rp"), ("l_ci", "icl_ci"), ("l_v", "icl_v"), ("diag_l", "icl_diag"),
               ("u_rp", "iclt_rp"), ("u_ci", "iclt_ci"), ("u_v", "iclt_v"))


@pytest.mark.parametrize("mat", ["cd", "sd"])
@pytest.mark.parametrize("sweeps,iters", [(3, 2), (1, 4)])
def test_chow_patel_golden(golden, mat, sweeps, iters):
    # detail::precondition's Neumann matrices and diagonals bit-exact, and both applies
    d = golden("chow_patel.npz")
    rp, ci, v = (d["cp"], d["cc"], d["cv"]) if mat == "cd" else (d["sp"], d["sc"], d["sv"])
    t = "%s_%d_%d_" % (mat, sweeps, iters)
    for fn, keys, z in ((oracle.chow_patel_ilu, CP_ILU_KEYS, "cp_ilu_z"),
                        (oracle.chow_patel_icc, CP_ICC_KEYS, "cp_icc_z")):
        F = fn(rp, ci, v, sweeps)
        for mine, ref in keys:
            assert np.array_equal(F[mine], d[t + ref]), (fn.__name__, mine)
        assert np.array_equal(oracle.chow_patel_apply(F, d["b_" + mat], iters), d[t + z])


def test_chow_patel_solves_golden(golden):
    # BiCGStab + chow_patel_ilu_precond and CG + chow_patel_icc_precond, default
    # tag (3 sweeps, 2 Jacobi iterations); single thread: identical iterations
    d = golden("chow_patel.npz")
    oracle.set_threads(1)
    try:
        x, it, err = oracle.solve("bicgstab", d["cp"], d["cc"], d["cv"], d["b_cd"], 1e-10, 2000,
                                  "cpilu")
        assert it == int(d["iters_bicgstab_cpilu"]) and err == float(d["error_bicgstab_cpilu"])
        assert rel_err(x, d["x_bicgstab_cpilu"]) < 1e-12
        x, it, err = oracle.solve("cg", d["sp"], d["sc"], d["sv"], d["b_sd"], 1e-10, 2000, "cpicc")
        assert it == int(d["iters_cg_cpicc"]) and err == float(d["error_cg_cpicc"])
        assert rel_err(x, d["x_cg_cpicc"]) < 1e-12
    finally:
        oracle.set_threads(oracle.max_threads())


@pytest.mark.parametrize("nb", [1, 8, 37])
def test_block_ilu_golden(golden, nb):
    # block_ilu_precond<compressed_matrix, ilu0_tag>: the blocks' factors
    # bit-exact; the apply bit-exact with the reference's skipped last column
    # of U reproduced, and different from it only through that column without
    d = golden("block_ilu.npz")
    B = oracle.block_ilu0(d["rp"], d["ci"], d["v"], num_blocks=nb)
    assert np.array_equal(B["lu"][:B["nnz"]], d["lu_%d" % nb])
    oracle.set_block_ilu_host_quirk(True)
    try:
        assert np.array_equal(oracle.block_ilu0_apply(B, d["b"]), d["z_%d" % nb])
    finally:
        oracle.set_block_ilu_host_quirk(False)
    z = oracle.block_ilu0_apply(B, d["b"])
    assert not np.array_equal(z, d["z_%d" % nb])
    # zeroing U's last column reproduces the reference exactly
    n = len(d["rp"]) - 1
    rows = np.repeat(np.arange(n), np.diff(B["rp"].astype(np.int64)))
    lu = B["lu"][:B["nnz"]].copy()
    lu[(B["ci"][:B["nnz"]] == n - 1) & (rows < n - 1)] = 0.0
    assert np.array_equal(oracle.block_ilu0_apply(dict(B, lu=lu), d["b"]), d["z_%d" % nb])


def test_block_ilu_solve_golden(golden):
    d = golden("block_ilu.npz")
    oracle.set_threads(1)
    oracle.set_block_ilu_host_quirk(True)
    try:
        x, it, err = oracle.solve("bicgstab", d["rp"], d["ci"], d["v"], d["b"], 1e-10, 2000, "bilu8")
        assert it == int(d["iters_bicgstab_bilu8"]) and err == float(d["error_bicgstab_bilu8"])
        assert rel_err(x, d["x_bicgstab_bilu8"]) < 1e-12
    finally:
        oracle.set_block_ilu_host_quirk(False)
        oracle.set_threads(oracle.max_threads())


MM_CASES = [("general", 1), ("general_case", 1), ("symmetric", 1), ("pattern", 1), ("complex", 1),
            ("zero_based", 0), ("extra_lines", 1), ("bad_word", 1), ("bad_field", 1),
            ("bad_symmetry", 1), ("array", 1), ("out_of_range", 1), ("too_few", 1),
            ("missing_value", 1)]


@pytest.mark.parametrize("name,base", MM_CASES)
def test_matrix_market_golden(golden, name, base):
    # io/matrix_market.hpp reader: lines read, the matrix, and which files fail
    d = golden("matrix_market.npz")
    path = os.path.join(os.path.dirname(__file__), "golden", "mm", name + ".mtx")
    ret = int(d[name + "__ret"][0])
    if ret == 0:
        with pytest.raises(ValueError):
            oracle.read_matrix_market(path, base)
        return
    lines, rows, cols, rp, ci, v = oracle.read_matrix_market(path, base)
    assert lines == ret and rows == int(d[name + "__ret"][1])
    assert np.array_equal(rp, d[name + "__rp"]) and np.array_equal(ci, d[name + "__ci"])
    assert np.array_equal(v, d[name + "__v"])


def test_cuthill_mckee_golden(golden):
    # misc/cuthill_mckee.hpp: both tags, two components and isolated nodes
    d = golden("cuthill_mckee.npz")
    for key, args in (("cm", (False, 0.0, 0)), ("acm_a0_g1", (True, 0.0, 1)),
                      ("acm_a05_g2", (True, 0.5, 2))):
        assert np.array_equal(oracle.cuthill_mckee(d["rp"], d["ci"], *args), d["perm_" + key]), key
    assert np.array_equal(oracle.cuthill_mckee(d["cp"], d["cc"]), d["perm_cd"])
    assert oracle.bandwidth(d["rp"], d["ci"]) == int(d["bw_cm"][0])


def test_spmv_f32_golden(golden):
    d = golden("spmv_f32_lognormal.npz")
    y = oracle.spmv_f32(d["rp"], d["ci"], d["v"].astype(np.float32), d["x"].astype(np.float32))
    assert rel_err(y, d["yf"]) < 1e-6


@pytest.mark.parametrize("name", ["formats_lognormal.npz", "formats_laplace2d.npz"])
def test_conversions_golden(golden, name):
    d = golden(name)
    rp, ci, v, x = d["rp"], d["ci"], d["v"], d["x"]
    n = len(rp) - 1
    w, coords, elems = oracle.ell(rp, ci, v)
    assert w == int(d["ell_width"][0])
    assert np.array_equal(coords, d["ell_coords"]) and np.array_equal(elems, d["ell_elems"])
    S = oracle.sell(rp, ci, v, C=int(d["C"]), sigma=1)
    for k, g in (("cpb", "sell_cpb"), ("bs", "sell_bs"), ("cols", "sell_cols"),
                 ("elems", "sell_elems")):
        assert np.array_equal(S[k], d[g]), k
    H = oracle.hyb(rp, ci, v, n, float(d["threshold"]))
    assert H["width"] == int(d["hyb_width"][0])
    assert max(H["tail_nnz"], 1) == int(d["hyb_tail_nnz"][0])
    assert np.array_equal(H["ell_coords"], d["hyb_ell_coords"])
    assert np.array_equal(H["ell_elems"], d["hyb_ell_elems"])
    assert np.array_equal(H["tail_rp"], d["hyb_tail_rp"])
    assert np.array_equal(H["tail_ci"], d["hyb_tail_ci"])
    assert np.array_equal(H["tail_v"], d["hyb_tail_v"])
    y = oracle.spmv(rp, ci, v, x)
    assert rel_err(y, d["y_ell"]) < 1e-14
    assert rel_err(y, d["y_hyb"]) < 1e-14
    if "y_sell" in d:
        assert rel_err(oracle.sell_spmv(S, n, int(d["C"]), x), d["y_sell"]) < 1e-14


def test_hyb_float_threshold_golden(golden):
    d = golden("hyb_f32_laplace2d.npz")
    n = len(d["rp"]) - 1
    H = oracle.hyb(d["rp"], d["ci"], d["v"], n, 0.8, is_float=True)
    assert H["width"] == int(d["width"][0])


@pytest.mark.parametrize("pc", ["none", "jacobi", "ilu0"])
def test_cg_golden(golden, pc):
    d = golden("cg_laplace2d.npz")
    x, it, err = oracle.solve("cg", d["rp"], d["ci"], d["v"], d["b"], float(d["tol"]),
                              int(d["max_iters"]), pc)
    assert it == int(d["iters_" + pc])
    assert abs(err - float(d["error_" + pc])) <= 1e-6 * float(d["error_" + pc])
    assert rel_err(x, d["x_" + pc]) < 1e-12


@pytest.mark.parametrize("pc", ["none", "jacobi"])
def test_bicgstab_golden(golden, pc):
    d = golden("bicgstab_convdiff.npz")
    x, it, err = oracle.solve("bicgstab", d["rp"], d["ci"], d["v"], d["b"], float(d["tol"]),
                              int(d["max_iters"]), pc)
    assert abs(it - int(d["iters_" + pc])) <= 1
    assert rel_err(x, d["x_" + pc]) < 1e-9


def test_gmres_golden_single_thread(golden):
    # the host stage-1 kernel drops vector tails depending on the thread count,
    # so this pin runs in a child process with one OpenMP thread and the
    # restatement's switch that reproduces that partition
    env = dict(os.environ, OMP_NUM_THREADS="1")
    code = (
        "import sys; sys.path.insert(0, %r); import oracle, numpy as np\n"
        "d = dict(np.load(%r))\n"
        "oracle.lib().vo_set_gmres_host_quirk(1)\n"
        "x, it, err = oracle.solve('gmres', d['rp'], d['ci'], d['v'], d['b'], 1e-10, 600, "
        "krylov_dim=30)\n"
        "assert it == int(d['iters']), (it, d['iters'])\n"
        "assert np.array_equal(x, d['x'])\n"
        "assert err == float(d['error'])\n") % (
        os.path.dirname(oracle.__file__),
        os.path.join(os.path.dirname(__file__), "golden", "gmres_convdiff_1thread.npz"))
    subprocess.run([sys.executable, "-c", code], env=env, check=True)


def test_gmres_converges_without_host_defect(golden):
    d = golden("gmres_convdiff_1thread.npz")
    x, it, err = oracle.solve("gmres", d["rp"], d["ci"], d["v"], d["b"], 1e-10, 600, krylov_dim=30)
    assert oracle.rel_residual(d["rp"], d["ci"], d["v"], x, d["b"]) < 2e-10
    assert it <= int(d["iters"])


def test_gmres_precond_golden_single_thread(golden):
    # the Householder GMRES restatement against the reference's own runs
    # (Jacobi, row scaling, ILU0, Chow-Patel ILU; Krylov dimensions 30, 10), one
    # OpenMP thread in both: iteration counts equal, x and the error estimate
    # bit-identical except with ILU0, whose level-scheduled apply sums in its
    # own order (x to 1e-15, the estimate near 1e-10 to 1e-4 relative)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    code = (
        "import sys; sys.path.insert(0, %r); import oracle, numpy as np\n"
        "d = dict(np.load(%r))\n"
        "for pc in ('jacobi', 'ilu0', 'row1', 'cpilu'):\n"
        "    for kd in (30, 10):\n"
        "        key = '%%s_%%d' %% (pc, kd)\n"
        "        x, it, err = oracle.solve('gmres', d['rp'], d['ci'], d['v'], d['b'], 1e-10, 1000,\n"
        "                                  pc, krylov_dim=kd)\n"
        "        assert it == int(d['iters_' + key]), (key, it, d['iters_' + key])\n"
        "        xr = d['x_' + key]\n"
        "        assert np.linalg.norm(x - xr) <= 1e-12 * np.linalg.norm(xr), key\n"
        "        assert abs(err - float(d['error_' + key])) <= 1e-4 * float(d['error_' + key]), key\n"
        "        if pc != 'ilu0':\n"
        "            assert np.array_equal(x, xr), key\n"
        "            assert err == float(d['error_' + key]), key\n") % (
        os.path.dirname(oracle.__file__),
        os.path.join(os.path.dirname(__file__), "golden", "gmres_precond_convdiff.npz"))
    subprocess.run([sys.executable, "-c", code], env=env, check=True)


def test_mixed_cg_golden(golden):
    d = golden("mixed_cg_laplace2d.npz")
    x, it, err = oracle.solve("mixed_cg", d["rp"], d["ci"], d["v"], d["b"], float(d["tol"]),
                              int(d["max_iters"]), inner_tol=float(d["inner_tol"]))
    assert it == int(d["iters"])
    assert rel_err(x, d["x"]) < 1e-12


def test_ilu0_golden(golden):
    d = golden("ilu0_convdiff.npz")
    rp, ci, v = d["rp"], d["ci"], d["v"]
    lu = oracle.ilu0_factor(rp, ci, v)
    assert np.array_equal(lu, d["lu"])  # same operation order, no FMA: bit-identical
    ud = oracle.diag(rp, ci, lu)
    assert np.array_equal(ud, d["udiag"])
    for tri, upper in (("L", False), ("U", True)):
        lv = oracle.level_setup(rp, ci, lu, ud, upper)
        assert np.array_equal(lv["level_ptr"], d[tri + "_level_ptr"])
        assert np.array_equal(lv["row_index"], d[tri + "_row_index"])
        assert np.array_equal(lv["row_ptr"], d[tri + "_row_ptr"])
        assert np.array_equal(lv["cols"], d[tri + "_cols"])
        assert np.array_equal(lv["vals"], d[tri + "_vals"])
    z = oracle.ilu0_apply(rp, ci, v, d["b"])
    assert rel_err(z, d["z"]) < 1e-14


def test_refined_cg_reaches_tolerance():
    import vclgb_gen as gen
    rp, ci, v, f = gen.diffusion3d(16, corr=3.0, contrast=1e3, seed=2)
    x, outer, inner, rr = oracle.refined_cg(rp, ci, v, f, tol=1e-10, inner_tol=1e-4)
    assert rr < 1e-10 and outer >= 2
    assert oracle.rel_residual(rp, ci, v, x, f) < 1e-10


@pytest.mark.skipif(not oracle.have_ref(), reason="ViennaCL tree not present here")
def test_live_reference_cg_jacobi_laplace256():
    # the reference's own CPU-runnable case: 256x256 Laplacian, Jacobi-PCG to 1e-8
    import vclgb_gen as gen
    rp, ci, v = gen.laplace2d(256, 256, scaled=True)
    b = gen.rhs_uniform(len(rp) - 1, 0)
    r = oracle.run_ref("cg", rp, ci, v, args=(1e-8, 2000, "jacobi"), b=b)
    x, it, err = oracle.solve("cg", rp, ci, v, b, 1e-8, 2000, "jacobi")
    assert abs(it - r["iters"]) <= 1
    assert rel_err(x, r["x"]) < 1e-10


def test_block_ilu_one_block_is_ilu0():
    # one block covering every row: block ILU0's factors are ILU0's, and its
    # column-sweep apply equals the level-scheduled apply up to rounding
    rp, ci, v = gen.convdiff2d(17, 13, peclet=8.0, shift=0.05)
    B = oracle.block_ilu0(rp, ci, v, num_blocks=1)
    assert np.array_equal(B["rp"], np.asarray(rp, np.uint32))
    assert np.array_equal(B["lu"][:B["nnz"]], oracle.ilu0_factor(rp, ci, v))
    b = gen.rhs_uniform(len(rp) - 1, 3)
    assert rel_err(oracle.block_ilu0_apply(B, b), oracle.ilu0_apply(rp, ci, v, b)) < 1e-14


def test_block_ilu_drops_couplings_between_blocks():
    # the block-diagonal pattern keeps exactly the entries whose row and column
    # share a block, in storage order
    rp, ci, v = gen.lognormal_random(500, mu=1.5, sigma=0.7, hi=40, seed=4)
    bounds = oracle.block_bounds(500, 7)
    B = oracle.block_ilu0(rp, ci, v, num_blocks=7)
    blk = np.zeros(500, np.int64)
    for i, (a, b) in enumerate(bounds):
        blk[a:b] = i
    rows = np.repeat(np.arange(500), np.diff(np.asarray(rp, np.int64)))
    keep = blk[rows] == blk[np.asarray(ci, np.int64)]
    assert np.array_equal(B["ci"][:B["nnz"]], np.asarray(ci)[keep])


def test_chow_patel_properties():
    # no sweep: L and U are A's scaled triangles (unit-modulus diagonals); the
    # ICC transpose holds L's entries; a matrix that is already triangular-free
    # (diagonal) makes the apply a division by the scaled diagonal
    rp, ci, v = gen.laplace2d(9, 7)
    n = len(rp) - 1
    F = oracle.chow_patel_ilu(rp, ci, v, 0)
    assert np.allclose(np.abs(F["diag_l"]), 1.0) and np.allclose(np.abs(F["diag_u"]), 1.0)
    G = oracle.chow_patel_icc(rp, ci, v, 2)
    assert len(G["u_ci"]) == len(G["l_ci"])
    lr = np.repeat(np.arange(n), np.diff(G["l_rp"].astype(np.int64)))
    ur = np.repeat(np.arange(n), np.diff(G["u_rp"].astype(np.int64)))
    assert sorted(zip(lr, G["l_ci"])) == sorted(zip(G["u_ci"], ur))
    drp, dci = np.arange(n + 1, dtype=np.uint32), np.arange(n, dtype=np.uint32)
    dv = np.linspace(2.0, 9.0, n)
    D = oracle.chow_patel_ilu(drp, dci, dv, 3)
    b = gen.rhs_uniform(n, 2)
    assert np.allclose(oracle.chow_patel_apply(D, b, 2), b / D["diag_l"] / D["diag_u"], rtol=1e-15)


@pytest.mark.parametrize("trans", [0, 1])
@pytest.mark.parametrize("tag", ["lower", "upper", "unit_lower", "unit_upper"])
@pytest.mark.parametrize("name", ["literal5", "convdiff_scaled", "lognormal"])
def test_inplace_solve_golden(golden, name, tag, trans):
    # the eight host triangular solves (host_based/sparse_matrix_operations.hpp:537-1090)
    # restated: bit-identical to the reference's outputs
    d = golden("trisolve.npz")
    z = oracle.inplace_solve(d[name + "_rp"], d[name + "_ci"], d[name + "_v"], d[name + "_b"],
                             tag, trans)
    assert np.array_equal(z, d["%s_tri_%s_%d" % (name, tag, trans)])


def test_gmres_clamp_false_convergence_and_restart_rule():
    # Jacobi GMRES(30) on the configured lognormal matrix (262,144 rows): the
    # reference's clamp of xi (gmres.hpp:575-578) ends the solve with an
    # estimate of 0 while the true residual is 2e-3; with the engine's rule (a
    # clamp ends the cycle, the next restart's residual decides) it converges
    rp, ci, v = gen.lognormal_random(262144, seed=1)
    b = gen.rhs_uniform(262144, 1)
    try:
        oracle.lib().vo_set_gmres_clamp_restart(0)
        x, it, err = oracle.solve("gmres", rp, ci, v, b, 1e-10, 3000, "jacobi", krylov_dim=30)
        assert err < 1e-10 and oracle.rel_residual(rp, ci, v, x, b) > 1e-3
        oracle.lib().vo_set_gmres_clamp_restart(1)
        x, it, err = oracle.solve("gmres", rp, ci, v, b, 1e-10, 3000, "jacobi", krylov_dim=30)
        assert err < 1e-10 and oracle.rel_residual(rp, ci, v, x, b) < 1e-8
    finally:
        oracle.lib().vo_set_gmres_clamp_restart(0)
