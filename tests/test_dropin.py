"""The drop-in boundary exercised from compiled code, not from Python:

* a ViennaCL program written against ViennaCL's own API only
  (tests/dropin/viennacl_dropin.cu: compressed_matrix, vector, prod, vector
  expressions, inner_prod, norm_2, element_prod, inplace_solve, solve with
  cg_tag / bicgstab_tag / gmres_tag and jacobi_precond) compiles against the
  shadow headers (viennacl-dev_gb300/shadow) placed before the ViennaCL tree,
  and every sparse, vector and solver call in it resolves to the engine's C
  ABI -- the object's undefined symbols are the engine's entry points.  The
  ViennaCL tree exists only where the oracle recipe finds it, so this test runs
  on the build machine (compile and link check; there is no GPU here);
* a plain C program (tests/dropin/abi_check.c) that includes only
  include/vclgb.h, built with gcc and run on the GPU, against the oracle."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

import oracle
from conftest import ROOT, iters_close, rel_err

DROPIN = os.path.join(ROOT, "tests", "dropin")
SHADOW = os.path.join(ROOT, "viennacl-dev_gb300", "shadow")
PKG = os.path.join(ROOT, "viennacl-dev_gb300")


def test_viennacl_program_routes_through_engine(tmp_path):
    tree = oracle.reference_tree()
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not tree or not os.path.exists(nvcc):
        pytest.skip("needs the ViennaCL source tree and nvcc")
    obj = str(tmp_path / "dropin.o")
    subprocess.run([nvcc, "-std=c++14", "-O0", "-DVIENNACL_WITH_CUDA", "-gencode",
                    "arch=compute_103a,code=sm_103a", "-I", SHADOW, "-I",
                    os.path.join(ROOT, "include"), "-I", tree, "-w", "-c", "-o", obj,
                    os.path.join(DROPIN, "viennacl_dropin.cu")], check=True)
    undefined = subprocess.run(["nm", "-u", obj], capture_output=True, text=True,
                               check=True).stdout
    used = {line.split()[-1] for line in undefined.splitlines() if "vclgb" in line}
    assert {"vclgbSpmv", "vclgbSolveCG", "vclgbSolveBiCGStab", "vclgbSolveGMRES",
            "vclgbJacobiCreate", "vclgbAvbv", "vclgbDot", "vclgbNorm2",
            "vclgbElementBinary", "vclgbCsrInplaceSolve", "vclgbCsrCreate"} <= used
    # and the program links against the library's exports
    lib = os.path.join(PKG, "libvclgb.so")
    if os.path.exists(lib):
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-o",
                        str(tmp_path / "dropin"), obj, "-L", PKG, "-lvclgb"], check=True)


@pytest.mark.gpu
def test_c_program_through_abi(tmp_path):
    exe = str(tmp_path / "abi_check")
    cuda = os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"))
    subprocess.run(["gcc", "-std=c99", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(cuda, "include"), "-o", exe, os.path.join(DROPIN, "abi_check.c"),
                    "-L", PKG, "-lvclgb", "-L", os.path.join(cuda, "lib64"), "-lcudart",
                    "-Wl,-rpath," + PKG + ":" + os.path.join(cuda, "lib64")], check=True)
    out = str(tmp_path / "out.f64")
    N = 40
    r = subprocess.run([exe, out, str(N)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    iters = int(r.stdout.split("iters")[1].split()[0])
    n = N * N
    res = np.fromfile(out, dtype=np.float64)
    y, x = res[:n], res[n:]
    # the same matrix and right-hand side, built here
    rows, cols, vals = [], [], []
    for j in range(N):
        for i in range(N):
            rr = j * N + i
            ent = []
            if j > 0:
                ent.append((rr - N, -1.0))
            if i > 0:
                ent.append((rr - 1, -1.0))
            ent.append((rr, 4.0))
            if i + 1 < N:
                ent.append((rr + 1, -1.0))
            if j + 1 < N:
                ent.append((rr + N, -1.0))
            for c, val in ent:
                rows.append(rr)
                cols.append(c)
                vals.append(val)
    rp = np.zeros(n + 1, np.uint32)
    np.cumsum(np.bincount(rows, minlength=n), out=rp[1:])
    ci, v = np.array(cols, np.uint32), np.array(vals)
    b = 1.0 + ((np.arange(n, dtype=np.uint64) * 7919) % 1000) / 1000.0
    assert rel_err(y, oracle.spmv(rp, ci, v, b)) < 1e-13
    xo, it_o, _ = oracle.solve("cg", rp, ci, v, b, 1e-10, 5000, "jacobi")
    assert iters_close(iters, it_o)
    assert rel_err(x, xo) < 1e-8
