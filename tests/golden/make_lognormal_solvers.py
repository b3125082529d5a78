"""Records what the oracle (the C restatement of ViennaCL's host backend) does on
the nonsymmetric lognormal matrices of the configured solver workload: row
lengths lognormal(mu=2.5, sigma=1.0) clipped to [1, 2000], uniform columns
without repeats, N(0,1) values and a diagonal of 1.1 times the row's absolute
sum, seed 1; rhs uniform [-1, 1], seed 1 (vclgb_gen.lognormal_random,
rhs_uniform).  Two sizes: 262,144 rows (the GPU tests compare against these
figures) and the full 4,194,304 rows.

Runs (tolerance 1e-10 unless stated), each with its iteration count, the
solver's own error estimate and the true relative residual ||b - Ax|| / ||b||:
  bicgstab_300, gmres30_300     no preconditioner (bicgstab.hpp:96-215 and
                                gmres.hpp:181-367), 300 iterations: both stall
  gmres30_jacobi_ref            Jacobi GMRES(30) as the reference runs it
                                (gmres.hpp:449-631): the clamp of xi ends the
                                solve as converged while the true residual is
                                large
  gmres30_jacobi_restart,       the same with the engine's rule (a clamp ends
  gmres30_jacobi_restart_1e-12  the cycle; the next restart's residual decides),
                                at tolerances 1e-10 and 1e-12
  bicgstab_jacobi_1e-12         Jacobi BiCGStab (bicgstab.hpp:398-489)
  bicgstab_3000, gmres30_3000   full size only: 3000 iterations, still stalled

Run from the repository root:
    python tests/golden/make_lognormal_solvers.py 262144     (about two minutes)
    python tests/golden/make_lognormal_solvers.py 4194304    (about an hour)
writes lognormal_<rows>_solvers.json beside this script.
"""
import json
import os
import sys
import time

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "viennacl-dev_gb300"))
import oracle  # noqa: E402
import vclgb_gen as gen  # noqa: E402


def main(n):
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                       "lognormal_%d_solvers.json" % n)
    t0 = time.time()
    rp, ci, v = gen.lognormal_random(n, seed=1)
    b = gen.rhs_uniform(n, 1)
    res = {"rows": n, "nnz": int(rp[-1]), "threads": oracle.max_threads(),
           "generate_s": time.time() - t0, "runs": {}}
    runs = [("bicgstab_300", "bicgstab", "none", 300, 1e-10, 0),
            ("gmres30_300", "gmres", "none", 300, 1e-10, 0),
            ("gmres30_jacobi_ref", "gmres", "jacobi", 3000, 1e-10, 0),
            ("gmres30_jacobi_restart", "gmres", "jacobi", 3000, 1e-10, 1),
            ("gmres30_jacobi_restart_1e-12", "gmres", "jacobi", 3000, 1e-12, 1),
            ("bicgstab_jacobi_1e-12", "bicgstab", "jacobi", 3000, 1e-12, 0)]
    if n > 1000000:
        runs += [("bicgstab_3000", "bicgstab", "none", 3000, 1e-10, 0),
                 ("gmres30_3000", "gmres", "none", 3000, 1e-10, 0)]
    for name, kind, pc, maxit, tol, clamp_restart in runs:
        oracle.lib().vo_set_gmres_clamp_restart(clamp_restart)
        t0 = time.time()
        x, it, err = oracle.solve(kind, rp, ci, v, b, tol, maxit, pc, krylov_dim=30)
        res["runs"][name] = {"iters": int(it), "error_estimate": float(err),
                             "true_rel_residual": float(oracle.rel_residual(rp, ci, v, x, b)),
                             "max_iters": maxit, "tol": tol, "seconds": time.time() - t0}
        print(name, res["runs"][name], flush=True)
        with open(out, "w") as f:
            json.dump(res, f, indent=1)
    oracle.lib().vo_set_gmres_clamp_restart(0)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 262144)
