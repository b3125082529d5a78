"""ctypes binding of liboracle.so -- the CPU restatement of ViennaCL's host
backend (vcl_oracle.c).  TEST INFRASTRUCTURE ONLY: imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline legs as the checker; the
GPU engine never imports it.

Also drives oracle/_ref/ref_driver (the reference's own host backend compiled
from its headers) where that binary exists.
"""
import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_U32, _SZ, _D, _I = ctypes.c_uint32, ctypes.c_size_t, ctypes.c_double, ctypes.c_int


class Tag(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("abs_tol", ctypes.c_double),
                ("max_iters", ctypes.c_uint32), ("krylov_dim", ctypes.c_uint32),
                ("max_iters_before_restart", ctypes.c_uint32), ("iters", ctypes.c_uint32),
                ("error", ctypes.c_double)]


class Precond(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("diag", ctypes.c_void_p), ("rp", ctypes.c_void_p),
                ("ci", ctypes.c_void_p), ("lu", ctypes.c_void_p), ("udiag", ctypes.c_void_p),
                ("l_rp", ctypes.c_void_p), ("l_ci", ctypes.c_void_p), ("l_v", ctypes.c_void_p),
                ("u_rp", ctypes.c_void_p), ("u_ci", ctypes.c_void_p), ("u_v", ctypes.c_void_p),
                ("jacobi_iters", ctypes.c_uint32)]


def reference_tree():
    """The ViennaCL source tree the recipe (Makefile) builds the reference driver
    against, or None where it is absent; REF=<path> in the environment overrides."""
    r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
    path = r.stdout.strip()
    return path if r.returncode == 0 and path else None


def build():
    """Compiles liboracle.so (and the reference driver where the reference exists)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if reference_tree():
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.vo_csr_spmv_d.argtypes = [_U32, _u32p, _u32p, _f64p, _f64p, _D, _D, _f64p]
        L.vo_csr_spmv_s.argtypes = [_U32, _u32p, _u32p, _f32p, _f32p, ctypes.c_float,
                                    ctypes.c_float, _f32p]
        L.vo_csr_spmv_strided_d.argtypes = [_U32, _u32p, _u32p, _f64p, _f64p, _SZ, _SZ, _D, _D,
                                            _f64p, _SZ, _SZ]
        L.vo_csr_diag_d.argtypes = [_U32, _u32p, _u32p, _f64p, _f64p]
        L.vo_row_norms_d.argtypes = [_U32, _u32p, _f64p, _U32, _f64p]
        L.vo_csr_row_blocks.argtypes = [_U32, _u32p, _u32p]
        L.vo_csr_row_blocks.restype = _SZ
        L.vo_ell_width.argtypes = [_U32, _u32p]
        L.vo_ell_width.restype = _U32
        L.vo_ell_fill_d.argtypes = [_U32, _u32p, _u32p, _f64p, _U32, _u32p, _f64p]
        L.vo_ell_spmv_d.argtypes = [_U32, _U32, _u32p, _f64p, _f64p, _D, _D, _f64p]
        L.vo_sell_layout.argtypes = [_U32, _u32p, _U32, _U32, _u32p, _u32p, _u32p]
        L.vo_sell_layout.restype = _SZ
        L.vo_sell_fill_d.argtypes = [_U32, _u32p, _u32p, _f64p, _U32, _u32p, _u32p, _u32p, _u32p,
                                     _f64p]
        L.vo_sell_spmv_d.argtypes = [_U32, _U32, _u32p, _u32p, _u32p, _u32p, _f64p, _f64p, _D, _D,
                                     _f64p]
        L.vo_hyb_width.argtypes = [_U32, _U32, _u32p, _D, _I, ctypes.POINTER(_SZ)]
        L.vo_hyb_width.restype = _U32
        L.vo_hyb_fill_d.argtypes = [_U32, _u32p, _u32p, _f64p, _U32, _u32p, _f64p, _u32p, _u32p,
                                    _f64p]
        L.vo_hyb_spmv_d.argtypes = [_U32, _U32, _u32p, _f64p, _u32p, _u32p, _f64p, _f64p, _D, _D,
                                    _f64p]
        L.vo_coo_fill_d.argtypes = [_U32, _u32p, _u32p, _f64p, _u32p, _f64p, _u32p]
        L.vo_coo_fill_d.restype = _SZ
        L.vo_coo_spmv_d.argtypes = [_U32, _SZ, _u32p, _f64p, _f64p, _D, _D, _f64p]
        for name in ("vo_cg_d", "vo_bicgstab_d"):
            getattr(L, name).argtypes = [_U32, _u32p, _u32p, _f64p, _f64p, _f64p,
                                         ctypes.POINTER(Tag), ctypes.POINTER(Precond)]
        L.vo_gmres_d.argtypes = [_U32, _u32p, _u32p, _f64p, _f64p, _f64p, ctypes.POINTER(Tag),
                                 ctypes.POINTER(Precond)]
        L.vo_mixed_cg_d.argtypes = [_U32, _u32p, _u32p, _f64p, _f64p, _f64p, ctypes.POINTER(Tag),
                                    ctypes.c_float]
        L.vo_ir_jacobi_d.argtypes = [_U32, _u32p, _u32p, _f64p, _f64p, _f64p, _D, _U32, _D, _U32,
                                     ctypes.POINTER(_U32), ctypes.POINTER(_U32),
                                     ctypes.POINTER(_D)]
        L.vo_ilu0_factor_d.argtypes = [_U32, _u32p, _u32p, _f64p]
        L.vo_cp_counts.argtypes = [_U32, _u32p, _u32p, ctypes.c_void_p, ctypes.c_void_p]
        L.vo_chow_patel_ilu_d.argtypes = [_U32, _u32p, _u32p, _f64p, _U32, _u32p, _u32p, _f64p,
                                          _f64p, _u32p, _u32p, _f64p, _f64p]
        L.vo_chow_patel_icc_d.argtypes = [_U32, _u32p, _u32p, _f64p, _U32, _u32p, _u32p, _f64p,
                                          _u32p, _u32p, _f64p, _f64p]
        L.vo_precond_apply_d.argtypes = [_U32, ctypes.c_void_p, _f64p]
        L.vo_block_ilu0_apply_d.argtypes = [_U32, _u32p, _u32p, _f64p, _f64p]
        L.vo_set_block_ilu_host_quirk.argtypes = [_I]
        L.vo_level_setup_d.argtypes = [_U32, _u32p, _u32p, _f64p, ctypes.c_void_p, _I,
                                       ctypes.POINTER(_SZ), ctypes.POINTER(_SZ), ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]
        L.vo_level_setup_d.restype = _SZ
        L.vo_level_substitute_d.argtypes = [_SZ, _u32p, _u32p, _u32p, _u32p, _f64p, _f64p]
        L.vo_dot_d.argtypes = [_SZ, _f64p, _f64p]
        L.vo_dot_d.restype = _D
        L.vo_rel_residual_d.argtypes = [_U32, _u32p, _u32p, _f64p, _f64p, _f64p]
        L.vo_rel_residual_d.restype = _D
        L.vo_csr_transpose_d.argtypes = [_U32, _U32, _u32p, _u32p, _f64p, _u32p, _u32p, _f64p,
                                         _u32p]
        L.vo_set_gmres_host_quirk.argtypes = [_I]
        L.vo_set_gmres_clamp_restart.argtypes = [_I]
        L.vo_csr_inplace_solve_d.argtypes = [_U32, _u32p, _u32p, _f64p, _f64p, _I, _I]
        L.vo_max_threads.restype = _I
        L.vo_set_threads.argtypes = [_I]
        _lib = L
    return _lib


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def set_threads(n):
    lib().vo_set_threads(int(n))


def max_threads():
    return lib().vo_max_threads()


def spmv(rp, ci, v, x, alpha=1.0, beta=0.0, y=None):
    n = len(rp) - 1
    y = np.zeros(n) if y is None else _c(y, np.float64).copy()
    lib().vo_csr_spmv_d(n, _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64),
                        _c(x, np.float64), alpha, beta, y)
    return y


def spmv_f32(rp, ci, v, x):
    n = len(rp) - 1
    y = np.zeros(n, np.float32)
    lib().vo_csr_spmv_s(n, _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float32),
                        _c(x, np.float32), 1.0, 0.0, y)
    return y


def spmv_strided(rp, ci, v, x, xs, xi, alpha, beta, y, ys, yi):
    n = len(rp) - 1
    y = _c(y, np.float64).copy()
    lib().vo_csr_spmv_strided_d(n, _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64),
                                _c(x, np.float64), xs, xi, alpha, beta, y, ys, yi)
    return y


def diag(rp, ci, v):
    n = len(rp) - 1
    d = np.zeros(n)
    lib().vo_csr_diag_d(n, _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64), d)
    return d


def row_norms(rp, v, norm):
    """row_scaling's diagonal: row norms (0 max, 1 sum, 2 Euclidean)."""
    n = len(rp) - 1
    d = np.zeros(n)
    lib().vo_row_norms_d(n, _c(rp, np.uint32), _c(v, np.float64), int(norm), d)
    return d


def row_blocks(rp):
    n = len(rp) - 1
    out = np.zeros(n + 1, np.uint32)
    k = lib().vo_csr_row_blocks(n, _c(rp, np.uint32), out)
    return out[:k + 1]


def ell(rp, ci, v):
    n = len(rp) - 1
    rp, ci, v = _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64)
    w = lib().vo_ell_width(n, rp)
    coords = np.zeros(max(n * w, 1), np.uint32)
    elems = np.zeros(max(n * w, 1))
    lib().vo_ell_fill_d(n, rp, ci, v, w, coords, elems)
    return w, coords[:n * w], elems[:n * w]


def sell(rp, ci, v, C=32, sigma=1):
    n = len(rp) - 1
    rp, ci, v = _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64)
    ns = (n - 1) // C + 1
    perm = np.zeros(n, np.uint32)
    cpb = np.zeros(ns, np.uint32)
    bs = np.zeros(ns, np.uint32)
    total = lib().vo_sell_layout(n, rp, C, sigma, perm, cpb, bs)
    cols = np.zeros(max(total, 1), np.uint32)
    elems = np.zeros(max(total, 1))
    lib().vo_sell_fill_d(n, rp, ci, v, C, perm, cpb, bs, cols, elems)
    return dict(perm=perm, cpb=cpb, bs=bs, cols=cols[:total], elems=elems[:total])


def sell_spmv(S, n, C, x):
    y = np.zeros(n)
    lib().vo_sell_spmv_d(n, C, S["perm"], S["cpb"], S["bs"], _c(S["cols"], np.uint32),
                         _c(S["elems"], np.float64), _c(x, np.float64), 1.0, 0.0, y)
    return y


def hyb(rp, ci, v, ncols, threshold=0.8, is_float=False):
    n = len(rp) - 1
    rp, ci, v = _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64)
    t = _SZ()
    w = lib().vo_hyb_width(n, ncols, rp, threshold, 1 if is_float else 0, ctypes.byref(t))
    tn = t.value
    ec = np.zeros(max(n * w, 1), np.uint32)
    ee = np.zeros(max(n * w, 1))
    trp = np.zeros(n + 1, np.uint32)
    tci = np.zeros(max(tn, 1), np.uint32)
    tv = np.zeros(max(tn, 1))
    lib().vo_hyb_fill_d(n, rp, ci, v, w, ec, ee, trp, tci, tv)
    return dict(width=w, ell_coords=ec[:n * w], ell_elems=ee[:n * w], tail_rp=trp,
                tail_ci=tci[:max(tn, 1)], tail_v=tv[:max(tn, 1)], tail_nnz=tn)


def coo(rp, ci, v):
    """coordinate_matrix copy: interleaved pairs, values (padded to 128), groups."""
    n = len(rp) - 1
    rp, ci, v = _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64)
    nnz = int(rp[-1])
    stored = (nnz + 127) // 128 * 128
    co = np.zeros(max(2 * stored, 2), np.uint32)
    el = np.zeros(max(stored, 1))
    gr = np.zeros(65, np.uint32)
    lib().vo_coo_fill_d(n, rp, ci, v, co, el, gr)
    return dict(coords=co[:2 * stored], elems=el[:stored], groups=gr, nnz=nnz, stored=stored)


def coo_spmv(n, C, x, alpha=1.0, beta=0.0, y0=None):
    y = np.zeros(n) if y0 is None else np.array(y0, dtype=np.float64)
    lib().vo_coo_spmv_d(n, C["nnz"], _c(C["coords"], np.uint32), _c(C["elems"], np.float64),
                        _c(x, np.float64), alpha, beta, y)
    return y


def _precond(kind, rp=None, ci=None, v=None):
    """kind: none | jacobi | ilu0 | row0/1/2 | cpilu[:sweeps:iters] | cpicc[:sweeps:iters]"""
    P = Precond()
    if kind.startswith("cp"):
        parts = kind.split(":")
        sweeps, iters = (int(parts[1]), int(parts[2])) if len(parts) == 3 else (3, 2)
        F = (chow_patel_ilu if parts[0] == "cpilu" else chow_patel_icc)(rp, ci, v, sweeps)
        return _cp_struct(F, iters)
    if kind.startswith("bilu"):
        B = block_ilu0(rp, ci, v, num_blocks=int(kind[4:]))
        P.kind = 4
        P.rp, P.ci, P.lu = B["rp"].ctypes.data, B["ci"].ctypes.data, B["lu"].ctypes.data
        return P, [B]
    P.kind = {"none": 0, "jacobi": 1, "ilu0": 2, "row0": 1, "row1": 1, "row2": 1}[kind]
    keep = []
    if kind == "jacobi" or kind.startswith("row"):
        d = diag(rp, ci, v) if kind == "jacobi" else row_norms(rp, v, int(kind[3]))
        keep.append(d)
        P.diag = d.ctypes.data
    elif kind == "ilu0":
        lu = _c(v, np.float64).copy()
        rp32, ci32 = _c(rp, np.uint32), _c(ci, np.uint32)
        lib().vo_ilu0_factor_d(len(rp) - 1, rp32, ci32, lu)
        keep += [lu, rp32, ci32]
        P.rp, P.ci, P.lu = rp32.ctypes.data, ci32.ctypes.data, lu.ctypes.data
    return P, keep


def solve(kind, rp, ci, v, b, tol, max_iters, precond="none", krylov_dim=30,
          max_before_restart=200, inner_tol=1e-2):
    """Runs cg / bicgstab / gmres / mixed_cg; returns (x, iters, error)."""
    n = len(rp) - 1
    rp, ci, v, b = _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64), _c(b, np.float64)
    x = np.zeros(n)
    t = Tag(tol=tol, abs_tol=0.0, max_iters=max_iters, krylov_dim=krylov_dim,
            max_iters_before_restart=max_before_restart)
    P, keep = _precond(precond, rp, ci, v)
    if kind == "cg":
        lib().vo_cg_d(n, rp, ci, v, b, x, ctypes.byref(t), ctypes.byref(P))
    elif kind == "bicgstab":
        lib().vo_bicgstab_d(n, rp, ci, v, b, x, ctypes.byref(t), ctypes.byref(P))
    elif kind == "gmres":
        lib().vo_gmres_d(n, rp, ci, v, b, x, ctypes.byref(t), ctypes.byref(P))
    elif kind == "mixed_cg":
        lib().vo_mixed_cg_d(n, rp, ci, v, b, x, ctypes.byref(t), inner_tol)
    else:
        raise ValueError(kind)
    del keep
    return x, t.iters, t.error


TRI_TAGS = {"lower": 0, "upper": 1, "unit_lower": 2, "unit_upper": 3}


def inplace_solve(rp, ci, v, vec, tag, trans=False):
    """inplace_solve(A or trans(A), vec, <tag>_tag) of the host backend; returns the result."""
    out = _c(vec, np.float64).copy()
    lib().vo_csr_inplace_solve_d(len(rp) - 1, _c(rp, np.uint32), _c(ci, np.uint32),
                                 _c(v, np.float64), out, TRI_TAGS[tag], int(bool(trans)))
    return out


def refined_cg(rp, ci, v, b, tol=1e-10, max_outer=30, inner_tol=1e-4, max_inner=100000):
    n = len(rp) - 1
    x = np.zeros(n)
    o, it, rr = _U32(), _U32(), _D()
    lib().vo_ir_jacobi_d(n, _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64),
                         _c(b, np.float64), x, tol, max_outer, inner_tol, max_inner,
                         ctypes.byref(o), ctypes.byref(it), ctypes.byref(rr))
    return x, o.value, it.value, rr.value


def rel_residual(rp, ci, v, x, b):
    return lib().vo_rel_residual_d(len(rp) - 1, _c(rp, np.uint32), _c(ci, np.uint32),
                                   _c(v, np.float64), _c(x, np.float64), _c(b, np.float64))


def ilu0_factor(rp, ci, v):
    lu = _c(v, np.float64).copy()
    lib().vo_ilu0_factor_d(len(rp) - 1, _c(rp, np.uint32), _c(ci, np.uint32), lu)
    return lu


def level_setup(rp, ci, lu, udiag, upper):
    n = len(rp) - 1
    rp, ci, lu = _c(rp, np.uint32), _c(ci, np.uint32), _c(lu, np.float64)
    ud = _c(udiag, np.float64)
    tr, tn = _SZ(), _SZ()
    nlev = lib().vo_level_setup_d(n, rp, ci, lu, ud.ctypes.data, int(upper), ctypes.byref(tr),
                                  ctypes.byref(tn), None, None, None, None, None)
    lp = np.zeros(nlev + 1, np.uint32)
    ri = np.zeros(max(tr.value, 1), np.uint32)
    rr = np.zeros(tr.value + 1, np.uint32)
    cc = np.zeros(max(tn.value, 1), np.uint32)
    vv = np.zeros(max(tn.value, 1))
    lib().vo_level_setup_d(n, rp, ci, lu, ud.ctypes.data, int(upper), ctypes.byref(tr),
                           ctypes.byref(tn), lp.ctypes.data, ri.ctypes.data, rr.ctypes.data,
                           cc.ctypes.data, vv.ctypes.data)
    return dict(level_ptr=lp, row_index=ri[:tr.value], row_ptr=rr, cols=cc[:tn.value],
                vals=vv[:tn.value])


def level_substitute(L, vec):
    vec = _c(vec, np.float64).copy()
    lib().vo_level_substitute_d(len(L["level_ptr"]) - 1, L["level_ptr"], L["row_index"],
                                L["row_ptr"], _c(L["cols"], np.uint32), _c(L["vals"], np.float64),
                                vec)
    return vec


def ilu0_apply(rp, ci, v, vec):
    """Level-scheduled ILU0 apply as ilu0_precond::apply with level scheduling."""
    lu = ilu0_factor(rp, ci, v)
    ud = diag(rp, ci, lu)
    L = level_setup(rp, ci, lu, ud, False)
    U = level_setup(rp, ci, lu, ud, True)
    z = level_substitute(L, vec)
    z = z / ud
    return level_substitute(U, z)


def block_bounds(n, num_blocks):
    """block_ilu_precond's default split (block_ilu.hpp:325-333): [i n / N, (i+1) n / N)."""
    return [((i * n) // num_blocks, ((i + 1) * n) // num_blocks) for i in range(num_blocks)]


def block_ilu0(rp, ci, v, bounds=None, num_blocks=8):
    """block_ilu_precond<compressed_matrix, ilu0_tag> setup (block_ilu.hpp:322-365,
    extract_block_matrix :69-113): A restricted to its diagonal blocks (entries
    whose column lies outside the row's block dropped, order kept), factorised by
    ILU0 -- the per-block factorisations, stored side by side."""
    n = len(rp) - 1
    bounds = block_bounds(n, num_blocks) if bounds is None else bounds
    rp64 = np.asarray(rp, np.int64)
    rows = np.repeat(np.arange(n), np.diff(rp64))
    lo, hi = np.zeros(n, np.int64), np.zeros(n, np.int64)
    for a, b in bounds:
        lo[a:b], hi[a:b] = a, b
    c = np.asarray(ci, np.int64)
    keep = (c >= lo[rows]) & (c < hi[rows])
    brp = np.zeros(n + 1, np.uint32)
    np.cumsum(np.bincount(rows[keep], minlength=n), out=brp[1:])
    bci = np.ascontiguousarray(np.asarray(ci, np.uint32)[keep])
    bv = np.asarray(v, np.float64)[keep]
    return {"rp": brp, "ci": bci if len(bci) else np.zeros(1, np.uint32),
            "lu": ilu0_factor(brp, bci, bv) if len(bv) else np.zeros(1), "nnz": int(keep.sum())}


def set_block_ilu_host_quirk(on):
    """Reproduce the reference apply's skipped last column of U (pinning only)."""
    lib().vo_set_block_ilu_host_quirk(int(bool(on)))


def block_ilu0_apply(B, vec):
    vec = _c(vec, np.float64).copy()
    lib().vo_block_ilu0_apply_d(len(vec), B["rp"], B["ci"], _c(B["lu"], np.float64), vec)
    return vec


def chow_patel_ilu(rp, ci, v, sweeps=3):
    """chow_patel_ilu_precond setup (chow_patel_ilu.hpp:110-150): the Neumann
    matrices I - D_L^-1 L and I - D_U^-1 U (diagonal entries kept as zeros) and
    D_L, D_U."""
    n = len(rp) - 1
    rp, ci, v = _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64)
    nl, nu = _SZ(), _SZ()
    lib().vo_cp_counts(n, rp, ci, ctypes.byref(nl), ctypes.byref(nu))
    F = dict(l_rp=np.zeros(n + 1, np.uint32), l_ci=np.zeros(max(nl.value, 1), np.uint32),
             l_v=np.zeros(max(nl.value, 1)), diag_l=np.zeros(max(n, 1)),
             u_rp=np.zeros(n + 1, np.uint32), u_ci=np.zeros(max(nu.value, 1), np.uint32),
             u_v=np.zeros(max(nu.value, 1)), diag_u=np.zeros(max(n, 1)))
    lib().vo_chow_patel_ilu_d(n, rp, ci, v, sweeps, F["l_rp"], F["l_ci"], F["l_v"], F["diag_l"],
                              F["u_rp"], F["u_ci"], F["u_v"], F["diag_u"])
    return _cp_trim(F, n, nl.value, nu.value)


def chow_patel_icc(rp, ci, v, sweeps=3):
    """chow_patel_icc_precond setup (chow_patel_ilu.hpp:77-107): I - D_L^-1 L,
    I - D_L^-1 L^T (as u_*) and D_L (as diag_l and diag_u)."""
    n = len(rp) - 1
    rp, ci, v = _c(rp, np.uint32), _c(ci, np.uint32), _c(v, np.float64)
    nl, nu = _SZ(), _SZ()
    lib().vo_cp_counts(n, rp, ci, ctypes.byref(nl), ctypes.byref(nu))
    m = max(nl.value, 1)
    F = dict(l_rp=np.zeros(n + 1, np.uint32), l_ci=np.zeros(m, np.uint32), l_v=np.zeros(m),
             u_rp=np.zeros(n + 1, np.uint32), u_ci=np.zeros(m, np.uint32), u_v=np.zeros(m),
             diag_l=np.zeros(max(n, 1)))
    lib().vo_chow_patel_icc_d(n, rp, ci, v, sweeps, F["l_rp"], F["l_ci"], F["l_v"], F["u_rp"],
                              F["u_ci"], F["u_v"], F["diag_l"])
    F["diag_u"] = F["diag_l"]
    return _cp_trim(F, n, nl.value, nl.value)


def _cp_trim(F, n, nl, nu):
    for k in ("l_ci", "l_v"):
        F[k] = F[k][:nl]
    for k in ("u_ci", "u_v"):
        F[k] = F[k][:nu]
    for k in ("diag_l", "diag_u"):
        F[k] = F[k][:n]
    return F


def _cp_struct(F, iters):
    P = Precond()
    P.kind = 3
    keep = {k: np.ascontiguousarray(a if len(a) else np.zeros(1, a.dtype)) for k, a in F.items()}
    P.diag, P.udiag = keep["diag_l"].ctypes.data, keep["diag_u"].ctypes.data
    for k in ("l_rp", "l_ci", "l_v", "u_rp", "u_ci", "u_v"):
        setattr(P, k, keep[k].ctypes.data)
    P.jacobi_iters = iters
    return P, [keep]


def chow_patel_apply(F, vec, jacobi_iters=2):
    """precond.apply(vec) of either Chow-Patel preconditioner (chow_patel_ilu.hpp:190-222,
    269-300)."""
    vec = _c(vec, np.float64).copy()
    P, keep = _cp_struct(F, jacobi_iters)
    lib().vo_precond_apply_d(len(vec), ctypes.byref(P), vec)
    del keep
    return vec


def strip_diagonal(rp, ci, v):
    """CSR without its diagonal entries (the Neumann matrices' zeroed diagonals)."""
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    keep = ci != rows
    nrp = np.zeros(n + 1, np.uint32)
    np.cumsum(np.bincount(rows[keep], minlength=n), out=nrp[1:])
    return nrp, ci[keep].astype(np.uint32), v[keep]


def transpose(nrows, ncols, rp, ci, v):
    nnz = int(rp[-1])
    trp = np.zeros(ncols + 1, np.uint32)
    tci = np.zeros(max(nnz, 1), np.uint32)
    tv = np.zeros(max(nnz, 1))
    mp = np.zeros(max(nnz, 1), np.uint32)
    lib().vo_csr_transpose_d(nrows, ncols, _c(rp, np.uint32), _c(ci, np.uint32),
                             _c(v, np.float64), trp, tci, tv, mp)
    return trp, tci[:nnz], tv[:nnz], mp[:nnz]


# ---- the reference's own host backend (oracle/_ref/ref_driver) ---------------
def have_ref():
    return os.path.exists(REF_DRIVER)


def run_ref(cmd, rp, ci, v, ncols=None, args=(), **vecs):
    """Runs ref_driver <cmd> on the arrays; returns a dict of its output files."""
    n = len(rp) - 1
    ncols = n if ncols is None else ncols
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, "meta.txt"), "w") as f:
            f.write("%d %d %d\n" % (n, ncols, int(rp[-1])))
        _c(rp, np.uint32).tofile(os.path.join(d, "rp.u32"))
        _c(ci, np.uint32).tofile(os.path.join(d, "ci.u32"))
        _c(v, np.float64).tofile(os.path.join(d, "v.f64"))
        for k, a in vecs.items():
            _c(a, np.float64).tofile(os.path.join(d, k + ".f64"))
        subprocess.run([REF_DRIVER, cmd, d] + [str(a) for a in args], check=True)
        out = {}
        for f in os.listdir(d):
            p = os.path.join(d, f)
            if f.endswith(".u32"):
                out[f[:-4]] = np.fromfile(p, np.uint32)
            elif f.endswith(".f64"):
                out[f[:-4]] = np.fromfile(p, np.float64)
            elif f.endswith(".f32"):
                out[f[:-4]] = np.fromfile(p, np.float32)
            elif f == "info.txt":
                it, err, sec = open(p).read().split()
                out["iters"], out["error"], out["seconds"] = int(it), float(err), float(sec)
        return out


# ---- io/matrix_market.hpp:101-326 (reader), restated in Python -------------
def read_matrix_market(path, index_base=1):
    """Follows read_matrix_market_file_impl: returns (lines_read, rows, cols,
    rp, ci, v) or raises ValueError where the reference returns 0.  Entries
    assign A(r, c) (and A(c, r) when symmetric); the later one wins."""
    symmetric = pattern = False
    header_done = False
    nnz = rows = cols = 0
    A = {}
    valid = 0
    linenum = 0
    with open(path, "rb") as f:
        raw = f.read().decode("latin-1").split("\n")
    if raw and raw[-1] == "":
        raw.pop()
    for text in raw:
        linenum += 1
        s = text.strip(" ")
        if s == "":
            continue
        if s[0] == "%":
            if s[1:2] != "%":
                continue
            words, tok = s[2:].split(), ""
            it = iter(words)

            def nxt():
                nonlocal tok
                tok = next(it, tok)  # a missing word keeps the previous one
                return tok.lower()
            if nxt() != "matrixmarket" or nxt() != "matrix":
                raise ValueError("header")
            kind = nxt()
            if kind != "coordinate":
                raise ValueError("array or unknown format")
            field = nxt()
            if field == "pattern":
                pattern = True
            elif field not in ("complex", "real"):
                raise ValueError("field")
            sym = nxt()
            if sym == "symmetric":
                symmetric = True
            elif sym != "general":
                raise ValueError("symmetry")
            continue
        w = s.split()
        if not header_done:
            if len(w) < 3:
                raise ValueError("size line")
            rows, cols, nnz = int(w[0]), int(w[1]), int(w[2])
            if rows == 0 or cols == 0:
                rows = cols = 0
            header_done = True
            if nnz == 0:
                break
            continue
        if len(w) < (2 if pattern else 3):
            raise ValueError("entry")
        r, c = int(w[0]) - index_base, int(w[1]) - index_base
        val = 1.0 if pattern else float(w[2])
        if not (0 <= r < rows) or not (0 <= c < cols):
            raise ValueError("index out of bounds")
        A[(r, c)] = val
        if symmetric:
            A[(c, r)] = val
        valid += 1
        if valid == nnz:
            break
    if not header_done or valid < nnz:
        raise ValueError("file ends early")
    keys = sorted(A)
    rp = np.zeros(rows + 1, np.uint32)
    for r, _ in keys:
        rp[r + 1] += 1
    rp = np.cumsum(rp).astype(np.uint32)
    ci = np.array([c for _, c in keys], np.uint32)
    v = np.array([A[k] for k in keys], np.float64)
    return linenum, rows, cols, rp, ci, v


# ---- misc/cuthill_mckee.hpp, restated in Python (small matrices) ------------
# Each node's unnumbered neighbours are ordered by degree with a stable sort;
# the reference's std::sort agrees with that whenever a node has at most 16
# such neighbours (its insertion-sort range), which holds for the stencil and
# banded test matrices used here.
def _cm_component(rp, ci, queue, done, perm, nxt):
    from collections import deque
    q = deque(queue)
    while q:
        node = q.popleft()
        if done[node]:
            continue
        perm[node] = nxt
        nxt += 1
        done[node] = True
        nb = [int(c) for c in ci[rp[node]:rp[node + 1]] if not done[c]]
        nb.sort(key=lambda c: rp[c + 1] - rp[c])
        q.extend(nb)
    return nxt


def cuthill_mckee(rp, ci, advanced=False, a=0.0, gmax=1):
    """reorder(matrix, cuthill_mckee_tag / advanced_cuthill_mckee_tag(a, gmax)):
    perm[i] = new label of node i (cuthill_mckee.hpp:366-421, 472-605)."""
    from collections import deque
    from itertools import combinations
    rp = np.asarray(rp, np.int64)
    ci = np.asarray(ci, np.int64)
    n = len(rp) - 1
    deg = np.diff(rp)
    perm = [0] * n
    done = [False] * n
    nxt = 0
    if not advanced:
        while nxt < n:
            root, found = 0, False
            for i in range(n):
                if done[i]:
                    continue
                if deg[i] == 1:
                    perm[i] = nxt
                    done[i] = True
                    nxt += 1
                    continue
                if not found or deg[i] < deg[root]:
                    root, found = i, True
            if not found:
                break
            nxt = _cm_component(rp, ci, [root], done, perm, nxt)
        return np.array(perm, np.uint32)

    def bw_of(done, perm):
        bw = 0
        for i in range(n):
            if not done[i]:
                continue
            cols = [perm[c] for c in ci[rp[i]:rp[i + 1]] if done[c]]
            if cols and max(cols) > min(cols):
                bw = max(bw, max(cols) - min(cols))
        return bw
    while nxt < n:
        start = next(i for i in range(n) if not done[i])
        comp, seen, q = [], [False] * n, deque([start])
        while q:
            v = q.popleft()
            if seen[v]:
                continue
            comp.append(v)
            seen[v] = True
            q.extend(int(c) for c in ci[rp[v]:rp[v + 1]] if c != v and not seen[c])
        dmin, dmax = min(deg[comp]), max(deg[comp])
        da = dmin + int(a * float(dmax - dmin))
        roots = [v for v in comp if deg[v] <= da]
        done0, perm0, nxt0 = list(done), list(perm), nxt
        best = None
        bw_best = 0
        for g in range(1, (len(roots) if gmax == 0 else min(gmax, len(roots))) + 1):
            for comb in combinations(range(len(roots)), g):
                d, p = list(done0), list(perm0)
                nxt = _cm_component(rp, ci, [roots[c] for c in comb], d, p, nxt0)
                bw = bw_of(d, p)
                if bw_best == 0 or bw < bw_best:
                    best, bw_best = (p, d), bw
        perm, done = list(best[0]), list(best[1])
    return np.array(perm, np.uint32)


def bandwidth(rp, ci):
    """max over rows of (largest - smallest column)."""
    bw = 0
    for i in range(len(rp) - 1):
        c = ci[rp[i]:rp[i + 1]]
        if len(c):
            bw = max(bw, int(c.max()) - int(c.min()))
    return bw
