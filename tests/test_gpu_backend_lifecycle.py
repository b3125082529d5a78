"""Backend lifetime through the C ABI: a backend on a stream of its own
(vclgbBackendCreate with NULL), solves that allocate the backend's loop and
reduction scratch, a move to the caller's stream (vclgbBackendSetStream), more
solves there, and destruction of the matrix, the preconditioner and the
backend in both orders -- all in one process, each solve checked against the
oracle."""
import ctypes

import numpy as np
import pytest

import oracle
import vclgb_gen as gen

pytestmark = pytest.mark.gpu


def _solve(V, lib, be, A, b, x, P):
    tag = V.SolverTag()
    lib.vclgbSolverTagInit(ctypes.byref(tag), 0)
    tag.tol = 1e-10
    tag.max_iters = 2000
    st = lib.vclgbSolveCG(be, A, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                          ctypes.byref(tag), P)
    return st, tag


def test_own_stream_then_caller_stream_then_destroy():
    import torch
    import vclgb as V
    torch.cuda.set_device(0)
    lib = V.load_library()
    rp, ci, v = gen.laplace2d(48)
    n, nnz = len(rp) - 1, int(rp[-1])
    d_rp = torch.tensor(rp.view(np.int32), device="cuda")
    d_ci = torch.tensor(ci.view(np.int32), device="cuda")
    d_v = torch.tensor(v, device="cuda")
    b_np = gen.rhs_uniform(n, 3)
    b = torch.tensor(b_np, device="cuda")
    x_ref, it_ref, _ = oracle.solve("cg", rp, ci, v, b_np, 1e-10, 2000, "jacobi")
    for rounds in range(2):  # a second backend after the first was destroyed
        torch.cuda.synchronize()
        be = ctypes.c_void_p()
        assert lib.vclgbBackendCreate(ctypes.byref(be), None) == V.SUCCESS
        A, P = ctypes.c_void_p(), ctypes.c_void_p()
        assert lib.vclgbCsrCreate(be, V.FLOAT64, n, n, nnz, ctypes.c_void_p(d_rp.data_ptr()),
                                  ctypes.c_void_p(d_ci.data_ptr()),
                                  ctypes.c_void_p(d_v.data_ptr()), ctypes.byref(A)) == V.SUCCESS
        assert lib.vclgbJacobiCreate(be, A, ctypes.byref(P)) == V.SUCCESS
        s = torch.cuda.Stream()
        for phase in ("own stream", "caller stream"):
            if phase == "caller stream":
                assert lib.vclgbBackendSetStream(be, ctypes.c_void_p(s.cuda_stream)) == V.SUCCESS
            x = torch.zeros(n, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            st, tag = _solve(V, lib, be, A, b, x, P)
            assert st == V.SUCCESS, (phase, lib.vclgbBackendLastError(be))
            assert lib.vclgbBackendSynchronize(be) == V.SUCCESS
            assert abs(tag.iters - it_ref) <= max(1, it_ref // 50), (phase, tag.iters, it_ref)
            assert oracle.rel_residual(rp, ci, v, x.cpu().numpy(), b_np) < 1e-9, phase
        if rounds == 0:  # objects first, then their backend
            assert lib.vclgbPrecondDestroy(ctypes.byref(P)) == V.SUCCESS
            assert lib.vclgbMatrixDestroy(ctypes.byref(A)) == V.SUCCESS
            assert lib.vclgbBackendDestroy(ctypes.byref(be)) == V.SUCCESS
        else:  # the backend first: the objects' buffers outlive its streams
            assert lib.vclgbBackendDestroy(ctypes.byref(be)) == V.SUCCESS
            assert lib.vclgbPrecondDestroy(ctypes.byref(P)) == V.SUCCESS
            assert lib.vclgbMatrixDestroy(ctypes.byref(A)) == V.SUCCESS
        assert not be.value and not A.value and not P.value
        s.synchronize()
