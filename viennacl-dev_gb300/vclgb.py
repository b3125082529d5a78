"""Python mirror of ViennaCL's sparse/solver API on top of the GB300 engine.

Names, argument meaning and results follow the reference so tests and
benchmarks read like ViennaCL code:

    A = compressed_matrix(row_ptr, cols, values, nrows, ncols)   # viennacl/compressed_matrix.hpp
    E = ell_matrix(A); S = sliced_ell_matrix(A, 32, 256); H = hyb_matrix(A)
    y = prod(A, x)                                               # viennacl/linalg/prod.hpp
    x = solve(A, b, cg_tag(1e-8, 2000), jacobi_precond(A))       # viennacl/linalg/cg.hpp
    tag.iters(), tag.error()

Every call goes through the C ABI of include/vclgb.h (libvclgb.so) with raw
device pointers; PyTorch only provides device memory and the current stream.
There is no CPU fallback: importing this module without the built library,
or using it without a CUDA device, raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libvclgb.so")

SUCCESS, GENERIC_FAILURE, INVALID_ARGUMENT, INVALID_MATRIX, OUT_OF_MEMORY, CUDA_ERROR, \
    NOT_CONVERGED, BREAKDOWN, ZERO_ON_DIAGONAL, TIMEOUT, UNSUPPORTED = range(11)
STATUS_NAMES = ["SUCCESS", "GENERIC_FAILURE", "INVALID_ARGUMENT", "INVALID_MATRIX",
                "OUT_OF_MEMORY", "CUDA_ERROR", "NOT_CONVERGED", "BREAKDOWN",
                "ZERO_ON_DIAGONAL", "TIMEOUT", "UNSUPPORTED"]
FLOAT32, FLOAT64 = 0, 1
CSR, ELL, SELL, HYB, COO = 0, 1, 2, 3, 4
FORMAT_NAMES = {CSR: "csr", ELL: "ell", SELL: "sell", HYB: "hyb", COO: "coo"}


class VclgbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES)
                                     else status, msg))
        self.status = status


class MatrixInfo(ctypes.Structure):
    _fields_ = [("format", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("rows", ctypes.c_uint32), ("cols", ctypes.c_uint32),
                ("nnz", ctypes.c_uint64), ("stored", ctypes.c_uint64),
                ("ell_width", ctypes.c_uint32), ("slice_height", ctypes.c_uint32),
                ("sigma", ctypes.c_uint32), ("num_slices", ctypes.c_uint32),
                ("tail_nnz", ctypes.c_uint64), ("num_bins", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class SolverTag(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("abs_tol", ctypes.c_double),
                ("max_iters", ctypes.c_uint32), ("krylov_dim", ctypes.c_uint32),
                ("max_iters_before_restart", ctypes.c_uint32), ("check_every", ctypes.c_uint32),
                ("iters", ctypes.c_uint32), ("status", ctypes.c_uint32),
                ("error", ctypes.c_double)]


class ScalarArg(ctypes.Structure):
    _fields_ = [("value", ctypes.c_double), ("d_value", ctypes.c_void_p),
                ("reciprocal", ctypes.c_int32), ("flip_sign", ctypes.c_int32)]


class TuneInfo(ctypes.Structure):
    _fields_ = [("format", ctypes.c_int32), ("slice_height", ctypes.c_uint32),
                ("sigma", ctypes.c_uint32), ("candidates", ctypes.c_uint32),
                ("csr_threshold", ctypes.c_double), ("us_csr", ctypes.c_double),
                ("us_best", ctypes.c_double)]


class ChowPatelInfo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("sweeps", ctypes.c_uint32),
                ("jacobi_iters", ctypes.c_uint32), ("nnz_L", ctypes.c_uint64),
                ("nnz_U", ctypes.c_uint64)]


class Ilu0Info(ctypes.Structure):
    _fields_ = [("num_levels_L", ctypes.c_uint32), ("num_levels_U", ctypes.c_uint32),
                ("rows_L", ctypes.c_uint64), ("rows_U", ctypes.c_uint64),
                ("nnz_L", ctypes.c_uint64), ("nnz_U", ctypes.c_uint64)]


_lib = None
_exiting = False  # set at interpreter exit: destructors then leave cleanup to process teardown
_P = ctypes.c_void_p


def _mark_exit():
    global _exiting
    _exiting = True


import atexit  # noqa: E402

atexit.register(_mark_exit)
_U32, _U64, _I64, _I32, _D, _F = (ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int64,
                                 ctypes.c_int, ctypes.c_double, ctypes.c_float)

# exported symbol -> (restype, argtypes); mirrors include/vclgb.h
SIGNATURES = {
    "vclgbVersion": (ctypes.c_char_p, []),
    "vclgbBackendCreate": (_I32, [ctypes.POINTER(_P), _P]),
    "vclgbBackendDestroy": (_I32, [ctypes.POINTER(_P)]),
    "vclgbBackendSetStream": (_I32, [_P, _P]),
    "vclgbBackendSynchronize": (_I32, [_P]),
    "vclgbBackendLastError": (ctypes.c_char_p, [_P]),
    "vclgbBackendLaunchCount": (_U64, [_P]),
    "vclgbBackendSetKernelTiming": (_I32, [_P, _I32]),
    "vclgbBackendKernelTimes": (_I32, [_P, _I32, ctypes.POINTER(ctypes.c_float), _U64,
                                       ctypes.POINTER(_U64)]),
    "vclgbCsrCreate": (_I32, [_P, _I32, _U32, _U32, _U32, _P, _P, _P, ctypes.POINTER(_P)]),
    "vclgbMatrixToEll": (_I32, [_P, _P, ctypes.POINTER(_P)]),
    "vclgbMatrixToSell": (_I32, [_P, _P, _U32, _U32, ctypes.POINTER(_P)]),
    "vclgbMatrixToHyb": (_I32, [_P, _P, _D, ctypes.POINTER(_P)]),
    "vclgbMatrixToCoo": (_I32, [_P, _P, ctypes.POINTER(_P)]),
    "vclgbMatrixToFloat32": (_I32, [_P, _P, ctypes.POINTER(_P)]),
    "vclgbEllWrap": (_I32, [_P, _I32, _U32, _U32, _U32, _P, _P, ctypes.POINTER(_P)]),
    "vclgbSellWrap": (_I32, [_P, _I32, _U32, _U32, _U32, _P, _P, _P, _P, ctypes.POINTER(_P)]),
    "vclgbHybWrap": (_I32, [_P, _I32, _U32, _U32, _U32, _P, _P, _P, _P, _P, _U64,
                            ctypes.POINTER(_P)]),
    "vclgbCooWrap": (_I32, [_P, _I32, _U32, _U32, _U64, _P, _P, ctypes.POINTER(_P)]),
    "vclgbReadMatrixMarket": (_I32, [_P, ctypes.c_char_p, _I64, _I32, ctypes.POINTER(_P),
                                     ctypes.POINTER(_U64)]),
    "vclgbWriteMatrixMarket": (_I32, [_P, _P, ctypes.c_char_p, _I64, _I32]),
    "vclgbCuthillMcKee": (_I32, [_P, _P, _I32, _D, _U64, _P]),
    "vclgbCsrPermute": (_I32, [_P, _P, _P, ctypes.POINTER(_P)]),
    "vclgbCsrBandwidth": (_I32, [_P, _P, ctypes.POINTER(_U32)]),
    "vclgbMatrixDestroy": (_I32, [ctypes.POINTER(_P)]),
    "vclgbMatrixGetInfo": (_I32, [_P, ctypes.POINTER(MatrixInfo)]),
    "vclgbMatrixExport": (_I32, [_P, _P, _I32, _P]),
    "vclgbCsrRowBlockCount": (_I32, [_P, _P, ctypes.POINTER(_U32)]),
    "vclgbSpmv": (_I32, [_P, _P, _D, _P, _I64, _I64, _D, _P, _I64, _I64]),
    "vclgbDot": (_I32, [_P, _I32, _U64, _P, _I64, _I64, _P, _I64, _I64, _P]),
    "vclgbNorm2": (_I32, [_P, _I32, _U64, _P, _I64, _I64, _P]),
    "vclgbJacobiCreate": (_I32, [_P, _P, ctypes.POINTER(_P)]),
    "vclgbRowScalingCreate": (_I32, [_P, _P, _U32, ctypes.POINTER(_P)]),
    "vclgbIlu0Create": (_I32, [_P, _P, _I32, ctypes.POINTER(_P)]),
    "vclgbPrecondApply": (_I32, [_P, _P, _P]),
    "vclgbCsrInplaceSolve": (_I32, [_P, _P, _I32, _I32, _P]),
    "vclgbMatrixAutotune": (_I32, [_P, _P, ctypes.POINTER(TuneInfo)]),
    "vclgbMatrixAutotuneClear": (_I32, [_P]),
    "vclgbAvbv": (_I32, [_P, _I32, _U64, _P, _I64, _I64, _P, _I64, _I64, ScalarArg, _P, _I64,
                         _I64, ScalarArg, _I32]),
    "vclgbElementBinary": (_I32, [_P, _I32, _U64, _P, _I64, _I64, _P, _I64, _I64, ScalarArg, _P,
                                  _I64, _I64, ScalarArg, _I32]),
    "vclgbElementUnary": (_I32, [_P, _I32, _U64, _P, _I64, _I64, _P, _I64, _I64, _I32]),
    "vclgbVectorAssign": (_I32, [_P, _I32, _U64, _P, _I64, _I64, _D]),
    "vclgbVectorSwap": (_I32, [_P, _I32, _U64, _P, _I64, _I64, _P, _I64, _I64]),
    "vclgbPrecondDestroy": (_I32, [ctypes.POINTER(_P)]),
    "vclgbIlu0GetInfo": (_I32, [_P, ctypes.POINTER(Ilu0Info)]),
    "vclgbIlu0Export": (_I32, [_P, _P, _I32, _P]),
    "vclgbBlockIlu0Create": (_I32, [_P, _P, _U32, _P, ctypes.POINTER(_P)]),
    "vclgbChowPatelIluCreate": (_I32, [_P, _P, _U32, _U32, ctypes.POINTER(_P)]),
    "vclgbChowPatelIccCreate": (_I32, [_P, _P, _U32, _U32, ctypes.POINTER(_P)]),
    "vclgbChowPatelGetInfo": (_I32, [_P, ctypes.POINTER(ChowPatelInfo)]),
    "vclgbChowPatelExport": (_I32, [_P, _P, _I32, _P]),
    "vclgbSolverTagInit": (None, [ctypes.POINTER(SolverTag), _I32]),
    "vclgbSolveCG": (_I32, [_P, _P, _P, _P, ctypes.POINTER(SolverTag), _P]),
    "vclgbSolveBiCGStab": (_I32, [_P, _P, _P, _P, ctypes.POINTER(SolverTag), _P]),
    "vclgbSolveGMRES": (_I32, [_P, _P, _P, _P, ctypes.POINTER(SolverTag), _P]),
    "vclgbSolveMixedCG": (_I32, [_P, _P, _P, _P, ctypes.POINTER(SolverTag), _F]),
    "vclgbSolveRefinedCG": (_I32, [_P, _P, _P, _P, ctypes.POINTER(SolverTag), _D, _U32,
                                   ctypes.POINTER(_U32)]),
    "vclgbBatchCreate": (_I32, [_P, _P, _U32, _P, _P, ctypes.POINTER(_P)]),
    "vclgbBatchTune": (_I32, [_P, _P, _P, ctypes.POINTER(ctypes.c_int32),
                              ctypes.POINTER(ctypes.c_int32)]),
    "vclgbBatchSolve": (_I32, [_P, _P, _P, _P, _D, _U32, _P, _P, _P]),
    "vclgbBatchDestroy": (_I32, [ctypes.POINTER(_P)]),
    "vclgbSolveAdjoint": (_I32, [_P, _P, _I32, _P, _P, _P, _P, _P, ctypes.POINTER(SolverTag),
                                 _I32]),
    "vclgbTransposeExport": (_I32, [_P, _P, _I32, _P]),
    "vclgbHybSpmvNoAlloc": (_I32, [_P, _I32, _U32, _U32, _P, _P, _P, _P, _P, _U64, _D, _P, _D,
                                   _P]),
}


def load_library(path=_LIB_PATH):
    """Loads libvclgb.so and declares every C-ABI signature (no GPU needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libvclgb.so is not built (run __graft_entry__.build()): %s" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("the GB300 engine needs a CUDA device; there is no CPU fallback")
    return torch


_backend = None


class Backend:
    """ViennaCLBackend: one stream, device scalars, error messages."""

    def __init__(self, stream=None):
        lib = load_library()
        torch = _torch()
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        h = _P()
        self._check_raw(lib.vclgbBackendCreate(ctypes.byref(h), _P(stream)), None)
        self.h = h
        self.lib = lib

    def _check_raw(self, st, h):
        if st != SUCCESS:
            msg = load_library().vclgbBackendLastError(h).decode() if h else ""
            raise VclgbError(st, msg)

    def check(self, st, allow=()):
        if st != SUCCESS and st not in allow:
            raise VclgbError(st, self.lib.vclgbBackendLastError(self.h).decode())
        return st

    def synchronize(self):
        self.check(self.lib.vclgbBackendSynchronize(self.h))

    def launches(self):
        return int(self.lib.vclgbBackendLaunchCount(self.h))

    def set_kernel_timing(self, enable):
        """Brackets every SpMV phase and fused vector pass with CUDA events."""
        self.check(self.lib.vclgbBackendSetKernelTiming(self.h, 1 if enable else 0))

    def kernel_times(self, kind, capacity=1 << 20):
        """Durations (ms) recorded since the last call: kind 0 SpMV, 1 vector pass."""
        buf = (ctypes.c_float * capacity)()
        cnt = _U64()
        self.check(self.lib.vclgbBackendKernelTimes(self.h, kind, buf, capacity, ctypes.byref(cnt)))
        return np.frombuffer(buf, dtype=np.float32, count=min(cnt.value, capacity)).copy()

    def __del__(self):
        if _exiting:
            return
        try:
            if getattr(self, "h", None):
                self.lib.vclgbBackendDestroy(ctypes.byref(self.h))
        except Exception:
            pass


def backend():
    """The process-wide default backend (created on first use)."""
    global _backend
    if _backend is None:
        _backend = Backend()
    return _backend


def _dtype_prec(dtype):
    torch = _torch()
    if dtype == torch.float64:
        return FLOAT64
    if dtype == torch.float32:
        return FLOAT32
    raise TypeError("only float32/float64 are supported")


def _dev(a, dtype):
    """numpy/torch -> contiguous CUDA tensor of dtype."""
    torch = _torch()
    if isinstance(a, np.ndarray):
        a = torch.from_numpy(np.ascontiguousarray(a))
    return a.to(device="cuda", dtype=dtype).contiguous()


def _ptr(t):
    return _P(t.data_ptr()) if t is not None and t.numel() else _P(0)


class _Matrix:
    fmt = None

    def __init__(self):
        self.h = None
        self.be = None
        self._keep = []

    def info(self):
        inf = MatrixInfo()
        self.be.check(self.be.lib.vclgbMatrixGetInfo(self.h, ctypes.byref(inf)))
        return inf

    def size1(self):
        return self.info().rows

    def size2(self):
        return self.info().cols

    def nnz(self):
        return self.info().nnz

    @property
    def dtype(self):
        torch = _torch()
        return torch.float64 if self.info().precision == FLOAT64 else torch.float32

    def export(self, which, count, dtype):
        torch = _torch()
        out = torch.empty(max(int(count), 1), dtype=dtype, device="cuda")
        self.be.check(self.be.lib.vclgbMatrixExport(self.be.h, self.h, which, _ptr(out)))
        return out[:int(count)]

    def __del__(self):
        if _exiting:
            return
        try:
            if self.h:
                self.be.lib.vclgbMatrixDestroy(ctypes.byref(self.h))
        except Exception:
            pass


class compressed_matrix(_Matrix):
    """viennacl::compressed_matrix wrapping device CSR arrays (uint32 indices)."""
    fmt = CSR

    def __init__(self, row_ptr, cols, values, nrows=None, ncols=None, dtype=None, be=None):
        super().__init__()
        torch = _torch()
        self.be = be or backend()
        if dtype is None:
            dtype = values.dtype if isinstance(values, torch.Tensor) else (
                torch.float64 if np.asarray(values).dtype == np.float64 else torch.float32)
            if isinstance(values, np.ndarray):
                dtype = torch.float64 if values.dtype == np.float64 else torch.float32
        rp = _dev(np.asarray(row_ptr, dtype=np.uint32).view(np.int32)
                  if not isinstance(row_ptr, torch.Tensor) else row_ptr, torch.int32)
        ci = _dev(np.asarray(cols, dtype=np.uint32).view(np.int32)
                  if not isinstance(cols, torch.Tensor) else cols, torch.int32)
        va = _dev(values, dtype)
        n = int(nrows if nrows is not None else rp.numel() - 1)
        m = int(ncols if ncols is not None else n)
        self.row_ptr, self.cols, self.values = rp, ci, va
        h = _P()
        self.be.check(self.be.lib.vclgbCsrCreate(self.be.h, _dtype_prec(dtype), n, m, int(va.numel()),
                                                 _ptr(rp), _ptr(ci), _ptr(va), ctypes.byref(h)))
        self.h = h

    def autotune(self):
        """Times the CSR kernel against SELL-C-sigma / HYB / ELL forms and keeps the
        fastest for every later product on this matrix; returns a dict of the choice."""
        info = TuneInfo()
        self.be.check(self.be.lib.vclgbMatrixAutotune(self.be.h, self.h, ctypes.byref(info)))
        return {"format": FORMAT_NAMES[info.format], "slice_height": info.slice_height,
                "sigma": info.sigma, "csr_threshold": info.csr_threshold,
                "candidates": info.candidates, "us_csr": info.us_csr, "us_best": info.us_best}

    def autotune_clear(self):
        """Drops the tuned form (products run on the CSR arrays again)."""
        self.be.check(self.be.lib.vclgbMatrixAutotuneClear(self.h))

    def row_blocks(self):
        torch = _torch()
        c = _U32()
        self.be.check(self.be.lib.vclgbCsrRowBlockCount(self.be.h, self.h, ctypes.byref(c)))
        return self.export(3, c.value + 1, torch.int32)


class _Converted(_Matrix):
    def __init__(self, src, fn, *args):
        super().__init__()
        if not isinstance(src, compressed_matrix):
            raise TypeError("conversions start from a compressed_matrix")
        self.be = src.be
        self._src = src  # the CSR arrays stay alive with the converted matrix
        h = _P()
        self.be.check(fn(self.be.h, src.h, *args, ctypes.byref(h)))
        self.h = h


class ell_matrix(_Converted):
    """viennacl::ell_matrix built on the GPU from a compressed_matrix."""
    fmt = ELL

    def __init__(self, csr):
        super().__init__(csr, load_library().vclgbMatrixToEll)


class sliced_ell_matrix(_Converted):
    """viennacl::sliced_ell_matrix (SELL-C-sigma) built on the GPU."""
    fmt = SELL

    def __init__(self, csr, rows_per_block=32, sigma=1):
        super().__init__(csr, load_library().vclgbMatrixToSell, int(rows_per_block), int(sigma))


class hyb_matrix(_Converted):
    """viennacl::hyb_matrix built on the GPU (csr_threshold as hyb_matrix.hpp:44)."""
    fmt = HYB

    def __init__(self, csr, csr_threshold=0.8):
        super().__init__(csr, load_library().vclgbMatrixToHyb, float(csr_threshold))


class coordinate_matrix(_Converted):
    """viennacl::coordinate_matrix<T, 128> built on the GPU from a
    compressed_matrix: interleaved (row, col) pairs, values, group boundaries."""
    fmt = COO

    def __init__(self, csr):
        super().__init__(csr, load_library().vclgbMatrixToCoo)


class _Wrapped(_Matrix):
    """A format already on the device in the reference layout, wrapped without
    copying; the tensors are kept alive with the handle."""

    def __init__(self, fmt, fn, arrays, *args, be=None):
        super().__init__()
        self.fmt = fmt
        self.be = be or backend()
        self._keep = list(arrays)
        h = _P()
        self.be.check(fn(self.be.h, *args, ctypes.byref(h)))
        self.h = h


def _u32_dev(a):
    torch = _torch()
    if isinstance(a, torch.Tensor):
        return a.to(device="cuda", dtype=torch.int32).contiguous()
    return _dev(np.asarray(a, dtype=np.uint32).view(np.int32), torch.int32)


def wrap_ell(rows, cols, width, coords, elems, be=None):
    """ell_matrix<T, 1> from its coords/elems buffers (rows*width each,
    column-major slots as ell_matrix.hpp lays them out)."""
    co, el = _u32_dev(coords), elems
    prec = _dtype_prec(el.dtype)
    return _Wrapped(ELL, load_library().vclgbEllWrap, (co, el), prec, int(rows), int(cols),
                    int(width), _ptr(co), _ptr(el), be=be)


def wrap_sliced_ell(rows, cols, slice_height, columns_per_block, column_indices, block_start,
                    elems, be=None):
    """sliced_ell_matrix<T, unsigned> (sigma 1) from its four buffers."""
    cpb, ci, bs, el = (_u32_dev(columns_per_block), _u32_dev(column_indices),
                       _u32_dev(block_start), elems)
    return _Wrapped(SELL, load_library().vclgbSellWrap, (cpb, ci, bs, el), _dtype_prec(el.dtype),
                    int(rows), int(cols), int(slice_height), _ptr(cpb), _ptr(ci), _ptr(bs),
                    _ptr(el), be=be)


def wrap_hyb(rows, cols, ell_width, ell_coords, ell_elems, tail_row_ptr, tail_cols, tail_vals,
             be=None):
    """hyb_matrix<T, 1> from its ELL part and CSR tail buffers."""
    co, trp, tci = _u32_dev(ell_coords), _u32_dev(tail_row_ptr), _u32_dev(tail_cols)
    el, tv = ell_elems, tail_vals
    return _Wrapped(HYB, load_library().vclgbHybWrap, (co, el, trp, tci, tv), _dtype_prec(el.dtype),
                    int(rows), int(cols), int(ell_width), _ptr(co), _ptr(el), _ptr(trp), _ptr(tci),
                    _ptr(tv), int(tv.numel()), be=be)


def wrap_coordinate(rows, cols, nnz, coords, elems, be=None):
    """coordinate_matrix<T, A> from its handle12 (interleaved (row, col)
    pairs, row-sorted) and handle buffers."""
    co, el = _u32_dev(coords), elems
    return _Wrapped(COO, load_library().vclgbCooWrap, (co, el), _dtype_prec(el.dtype), int(rows),
                    int(cols), int(nnz), _ptr(co), _ptr(el), be=be)


class _Loaded(compressed_matrix):
    """A compressed_matrix whose device arrays the library owns (file reader)."""

    def __init__(self, h, be):
        _Matrix.__init__(self)
        self.be, self.h = be, h


def read_matrix_market_file(path, index_base=1, dtype=None, be=None):
    """io::read_matrix_market_file: returns (compressed_matrix, lines read).
    Raises VclgbError (INVALID_ARGUMENT, the cause in the message) where the
    reference prints an error and returns 0."""
    torch = _torch()
    be = be or backend()
    h = _P()
    lines = _U64()
    prec = _dtype_prec(dtype or torch.float64)
    be.check(be.lib.vclgbReadMatrixMarket(be.h, os.fsencode(path), int(index_base), prec,
                                          ctypes.byref(h), ctypes.byref(lines)))
    return _Loaded(h, be), int(lines.value)


def write_matrix_market_file(A, path, index_base=1, digits=0):
    """io::write_matrix_market_file for a compressed_matrix (digits 0 = the
    reference's 6 significant digits)."""
    A.be.check(A.be.lib.vclgbWriteMatrixMarket(A.be.h, A.h, os.fsencode(path), int(index_base),
                                               int(digits)))


class cuthill_mckee_tag:
    """reorder(matrix, cuthill_mckee_tag())."""
    advanced, a, gmax = 0, 0.0, 1


class advanced_cuthill_mckee_tag:
    """advanced_cuthill_mckee_tag(a, gmax): root candidates of degree at most
    deg_min + a (deg_max - deg_min), up to gmax roots at once."""
    advanced = 1

    def __init__(self, a=0.0, gmax=1):
        self.a, self.gmax = float(a), int(gmax)


def reorder(A, tag):
    """viennacl::reorder on a compressed_matrix: device uint32 tensor with
    perm[i] = new label of node i."""
    torch = _torch()
    perm = torch.empty(max(A.size1(), 1), dtype=torch.int32, device="cuda")
    A.be.check(A.be.lib.vclgbCuthillMcKee(A.be.h, A.h, tag.advanced, tag.a, tag.gmax, _ptr(perm)))
    return perm[:A.size1()]


def permute(A, perm):
    """P A P^T as a new compressed_matrix (B(perm[i], perm[j]) = A(i, j))."""
    p = _u32_dev(perm)
    h = _P()
    A.be.check(A.be.lib.vclgbCsrPermute(A.be.h, A.h, _ptr(p), ctypes.byref(h)))
    return _Loaded(h, A.be)


def bandwidth(A):
    """max over rows of (largest - smallest column index)."""
    bw = _U32()
    A.be.check(A.be.lib.vclgbCsrBandwidth(A.be.h, A.h, ctypes.byref(bw)))
    return int(bw.value)


def prod(A, x, alpha=1.0, y=None, beta=0.0, x_start=0, x_stride=1, y_start=0, y_stride=1,
         y_size=None):
    """linalg::prod_impl(A, x, alpha, y, beta): y = alpha*A*x + beta*y on the GPU."""
    torch = _torch()
    dt = A.dtype
    x = x if (isinstance(x, torch.Tensor) and x.is_cuda and x.dtype == dt) else _dev(x, dt)
    if y is None:
        y = torch.empty(y_size or A.size1(), dtype=dt, device="cuda")
    A.be.check(A.be.lib.vclgbSpmv(A.be.h, A.h, float(alpha), _ptr(x), x_start, x_stride,
                                  float(beta), _ptr(y), y_start, y_stride))
    return y


# ---- triangular solves: linalg::inplace_solve(A | trans(A), vec, tag) --------
class lower_tag:
    """viennacl::linalg::lower_tag"""
    code = 0


class upper_tag:
    """viennacl::linalg::upper_tag"""
    code = 1


class unit_lower_tag:
    """viennacl::linalg::unit_lower_tag"""
    code = 2


class unit_upper_tag:
    """viennacl::linalg::unit_upper_tag"""
    code = 3


class trans:
    """viennacl::trans(A): the transposed operand of inplace_solve."""

    def __init__(self, A):
        self.A = A


def inplace_solve(A, vec, tag):
    """linalg::inplace_solve(A, vec, tag) / inplace_solve(trans(A), vec, tag) for a
    compressed_matrix: vec (a contiguous CUDA tensor of the matrix precision) is
    overwritten by the solution of the tag's triangle; returns vec."""
    torch = _torch()
    transposed = isinstance(A, trans)
    M = A.A if transposed else A
    if not (isinstance(vec, torch.Tensor) and vec.is_cuda and vec.dtype == M.dtype
            and vec.is_contiguous()):
        raise VclgbError(INVALID_ARGUMENT, "inplace_solve needs a contiguous CUDA vector "
                         "of the matrix precision")
    code = tag.code if hasattr(tag, "code") else int(tag)
    M.be.check(M.be.lib.vclgbCsrInplaceSolve(M.be.h, M.h, code, int(transposed), _ptr(vec)))
    return vec


# ---- vector updates and element-wise operations -----------------------------
# Vectors are CUDA tensors of one precision; a strided view is given as
# (tensor, start, stride) with the element count n.
def _vec(v):
    """tensor | (tensor, start, stride) -> (tensor, start, stride)"""
    if isinstance(v, tuple):
        return v[0], int(v[1]), int(v[2])
    return v, 0, 1


def _scalar(a, reciprocal=False, flip_sign=False):
    """a host number or a 0-d CUDA tensor (viennacl::scalar) -> ScalarArg"""
    torch = _torch()
    if isinstance(a, torch.Tensor):
        return ScalarArg(0.0, a.data_ptr(), int(reciprocal), int(flip_sign)), a
    return ScalarArg(float(a), None, int(reciprocal), int(flip_sign)), None


def _count(t, start, stride, n):
    return int(n) if n is not None else (t.numel() - start + abs(stride) - 1) // abs(stride)


def avbv(y, x, alpha, z=None, beta=0.0, accumulate=False, n=None, reciprocal_alpha=False,
         flip_sign_alpha=False, reciprocal_beta=False, flip_sign_beta=False, be=None):
    """linalg av / avbv / avbv_v: y = x*alpha [+ z*beta], or y += ... (accumulate);
    alpha/beta host numbers or device scalars, divided by when reciprocal_*."""
    be = be or backend()
    (ty, ys, yi), (tx, xs, xi) = _vec(y), _vec(x)
    sa, keep_a = _scalar(alpha, reciprocal_alpha, flip_sign_alpha)
    sb, keep_b = _scalar(beta, reciprocal_beta, flip_sign_beta)
    tz, zs, zi = _vec(z) if z is not None else (None, 0, 1)
    be.check(be.lib.vclgbAvbv(be.h, _dtype_prec(ty.dtype), _count(ty, ys, yi, n), _ptr(ty), ys, yi,
                              _ptr(tx), xs, xi, sa, _ptr(tz), zs, zi, sb, int(bool(accumulate))))
    return ty


def av(y, x, alpha, **kw):
    """linalg av: y = x*alpha (x/alpha with reciprocal_alpha=True)."""
    return avbv(y, x, alpha, **kw)


def _binary(op, x, z, out, n, be):
    torch = _torch()
    be = be or backend()
    xv = _vec(x) if isinstance(x, (torch.Tensor, tuple)) else None
    zv = _vec(z) if isinstance(z, (torch.Tensor, tuple)) else None
    ref = (xv or zv)[0]
    if out is None:
        out = torch.empty(_count(*(xv or zv), n), dtype=ref.dtype, device="cuda")
    ty, ys, yi = _vec(out)
    sx, kx = _scalar(x) if xv is None else (ScalarArg(), None)
    sz, kz = _scalar(z) if zv is None else (ScalarArg(), None)
    xv = xv or (None, 0, 1)
    zv = zv or (None, 0, 1)
    be.check(be.lib.vclgbElementBinary(be.h, _dtype_prec(ty.dtype), _count(ty, ys, yi, n), _ptr(ty),
                                       ys, yi, _ptr(xv[0]), xv[1], xv[2], sx, _ptr(zv[0]), zv[1],
                                       zv[2], sz, op))
    return ty


def element_prod(x, z, out=None, n=None, be=None):
    """element_prod(x, z) (either may be a scalar)."""
    return _binary(0, x, z, out, n, be)


def element_div(x, z, out=None, n=None, be=None):
    """element_div(x, z) (either may be a scalar)."""
    return _binary(1, x, z, out, n, be)


def element_pow(x, z, out=None, n=None, be=None):
    """element_pow(x, z) (either may be a scalar)."""
    return _binary(2, x, z, out, n, be)


UNARY_OPS = ["abs", "acos", "acosh", "asin", "asinh", "atan", "atanh", "ceil", "cos", "cosh",
             "erf", "erfc", "exp", "exp2", "exp10", "fabs", "floor", "log", "log2", "log10",
             "round", "sin", "sinh", "sqrt", "tan", "tanh", "trunc", "rsqrt", "sign"]


def element_unary(name, x, out=None, n=None, be=None):
    """element_<name>(x) for the reference's unary element functions."""
    torch = _torch()
    be = be or backend()
    tx, xs, xi = _vec(x)
    if out is None:
        out = torch.empty(_count(tx, xs, xi, n), dtype=tx.dtype, device="cuda")
    ty, ys, yi = _vec(out)
    be.check(be.lib.vclgbElementUnary(be.h, _dtype_prec(ty.dtype), _count(ty, ys, yi, n), _ptr(ty),
                                      ys, yi, _ptr(tx), xs, xi, 16 + UNARY_OPS.index(name)))
    return ty


def vector_assign(y, alpha, n=None, be=None):
    """vector_assign: y = alpha."""
    be = be or backend()
    ty, ys, yi = _vec(y)
    be.check(be.lib.vclgbVectorAssign(be.h, _dtype_prec(ty.dtype), _count(ty, ys, yi, n), _ptr(ty),
                                      ys, yi, float(alpha)))
    return ty


def vector_swap(x, y, n=None, be=None):
    """vector_swap: exchanges the elements of x and y."""
    be = be or backend()
    (tx, xs, xi), (ty, ys, yi) = _vec(x), _vec(y)
    be.check(be.lib.vclgbVectorSwap(be.h, _dtype_prec(tx.dtype), _count(tx, xs, xi, n), _ptr(tx),
                                    xs, xi, _ptr(ty), ys, yi))


def inner_prod(x, y, be=None):
    """linalg::inner_prod -> device scalar (0-d tensor)."""
    torch = _torch()
    be = be or backend()
    out = torch.empty((), dtype=x.dtype, device="cuda")
    be.check(be.lib.vclgbDot(be.h, _dtype_prec(x.dtype), x.numel(), _ptr(x), 0, 1, _ptr(y), 0, 1,
                             _ptr(out)))
    return out


def norm_2(x, be=None):
    """linalg::norm_2 -> device scalar (0-d tensor)."""
    torch = _torch()
    be = be or backend()
    out = torch.empty((), dtype=x.dtype, device="cuda")
    be.check(be.lib.vclgbNorm2(be.h, _dtype_prec(x.dtype), x.numel(), _ptr(x), 0, 1, _ptr(out)))
    return out


# ---- tags -------------------------------------------------------------------
class _Tag:
    kind = 0

    def __init__(self, tol, max_iterations, krylov_dim=0, max_before_restart=0, check_every=0):
        self.t = SolverTag()
        load_library().vclgbSolverTagInit(ctypes.byref(self.t), self.kind)
        self.t.tol = tol
        self.t.max_iters = max_iterations
        if krylov_dim:
            self.t.krylov_dim = krylov_dim
        if max_before_restart:
            self.t.max_iters_before_restart = max_before_restart
        self.t.check_every = check_every

    def tolerance(self):
        return self.t.tol

    def abs_tolerance(self, v=None):
        if v is not None and v >= 0:
            self.t.abs_tol = v
        return self.t.abs_tol

    def max_iterations(self):
        return self.t.max_iters

    def iters(self):
        return self.t.iters

    def error(self):
        return self.t.error

    def status(self):
        return self.t.status


class cg_tag(_Tag):
    kind = 0

    def __init__(self, tol=1e-8, max_iterations=300, check_every=0):
        super().__init__(tol, max_iterations, check_every=check_every)


class bicgstab_tag(_Tag):
    kind = 1

    def __init__(self, tol=1e-8, max_iters=400, max_iters_before_restart=200, check_every=0):
        super().__init__(tol, max_iters, max_before_restart=max_iters_before_restart,
                         check_every=check_every)


class gmres_tag(_Tag):
    kind = 2

    def __init__(self, tol=1e-10, max_iterations=300, krylov_dim=20):
        super().__init__(tol, max_iterations, krylov_dim=krylov_dim)


class mixed_precision_cg_tag(_Tag):
    kind = 0

    def __init__(self, tol=1e-8, max_iterations=300, inner_tol=1e-2):
        super().__init__(tol, max_iterations)
        self.inner_tol = inner_tol


class refined_cg_tag(_Tag):
    """FP64 iterative refinement around FP32 Jacobi-PCG inner solves (new form)."""
    kind = 0

    def __init__(self, tol=1e-10, max_iterations=100000, inner_tol=1e-4, max_outer=30):
        super().__init__(tol, max_iterations)
        self.inner_tol = inner_tol
        self.max_outer = max_outer
        self.outer = 0


# ---- preconditioners ----------------------------------------------------------
class _Precond:
    def __init__(self, A, fn, *args):
        self.be = A.be
        self._A = A
        h = _P()
        self.be.check(fn(self.be.h, A.h, *args, ctypes.byref(h)))
        self.h = h

    def apply(self, vec):
        self.be.check(self.be.lib.vclgbPrecondApply(self.be.h, self.h, _ptr(vec)))
        return vec

    def __del__(self):
        if _exiting:
            return
        try:
            if self.h:
                self.be.lib.vclgbPrecondDestroy(ctypes.byref(self.h))
        except Exception:
            pass


class jacobi_precond(_Precond):
    """jacobi_precond<compressed_matrix>(A, jacobi_tag())."""

    def __init__(self, A, tag=None):
        super().__init__(A, load_library().vclgbJacobiCreate)


class row_scaling_tag:
    """row_scaling_tag(p): 0 = max norm, 1 = sum norm, 2 = Euclidean norm of each row."""

    def __init__(self, p=2):
        self.p = int(p)

    def norm(self):
        return self.p


class row_scaling(_Precond):
    """row_scaling<compressed_matrix>(A, row_scaling_tag(p)): divides by row norms."""

    def __init__(self, A, tag=None):
        super().__init__(A, load_library().vclgbRowScalingCreate,
                         (tag or row_scaling_tag()).norm())


class ilu0_precond(_Precond):
    """ilu0_precond<compressed_matrix>(A, ilu0_tag(use_level_scheduling))."""

    def __init__(self, A, use_level_scheduling=True):
        super().__init__(A, load_library().vclgbIlu0Create, 1 if use_level_scheduling else 0)

    def info(self):
        inf = Ilu0Info()
        self.be.check(self.be.lib.vclgbIlu0GetInfo(self.h, ctypes.byref(inf)))
        return inf

    def levels(self):
        return self.info().num_levels_L

    def export(self, which, count, dtype):
        torch = _torch()
        out = torch.empty(max(int(count), 1), dtype=dtype, device="cuda")
        self.be.check(self.be.lib.vclgbIlu0Export(self.be.h, self.h, which, _ptr(out)))
        return out[:int(count)]


class block_ilu_precond(ilu0_precond):
    """block_ilu_precond<compressed_matrix, ilu0_tag>(A, ilu0_tag(), num_blocks) or
    (A, ilu0_tag(), block_boundaries=[(start, stop), ...])."""

    def __init__(self, A, tag=None, num_blocks=8, block_boundaries=None):
        if block_boundaries is not None:
            num_blocks = len(block_boundaries)
            self._bounds = np.ascontiguousarray(
                np.asarray(block_boundaries, dtype=np.uint32).reshape(-1))
            bp = _P(self._bounds.ctypes.data) if self._bounds.size else _P(0)
        else:
            bp = _P(0)
        self.num_blocks = int(num_blocks)
        _Precond.__init__(self, A, load_library().vclgbBlockIlu0Create, int(num_blocks), bp)


class chow_patel_tag:
    """chow_patel_tag(num_sweeps=3, num_jacobi_iters=2) (chow_patel_ilu.hpp:44-70)."""

    def __init__(self, num_sweeps=3, num_jacobi_iters=2):
        self._sweeps = int(num_sweeps)
        self._iters = int(num_jacobi_iters)

    def sweeps(self, num=None):
        if num is None:
            return self._sweeps
        self._sweeps = int(num)

    def jacobi_iters(self, num=None):
        if num is None:
            return self._iters
        self._iters = int(num)


class _ChowPatel(_Precond):
    _create = None

    def __init__(self, A, tag=None):
        tag = tag or chow_patel_tag()
        super().__init__(A, getattr(load_library(), self._create), tag.sweeps(),
                         tag.jacobi_iters())

    def info(self):
        inf = ChowPatelInfo()
        self.be.check(self.be.lib.vclgbChowPatelGetInfo(self.h, ctypes.byref(inf)))
        return inf

    def export(self, which):
        """0..3: L row_ptr, cols, values (I - D_L^-1 L without its diagonal), D_L;
        4..7: the same for U (ICC: L^T)."""
        torch = _torch()
        inf = self.info()
        n = self._A.size1()
        count = [n + 1, inf.nnz_L, inf.nnz_L, n, n + 1, inf.nnz_U, inf.nnz_U, n][which]
        dtype = torch.int32 if which % 4 in (0, 1) else self._A.dtype
        out = torch.empty(max(int(count), 1), dtype=dtype, device="cuda")
        self.be.check(self.be.lib.vclgbChowPatelExport(self.be.h, self.h, which, _ptr(out)))
        return out[:int(count)]


class chow_patel_ilu_precond(_ChowPatel):
    """chow_patel_ilu_precond<compressed_matrix>(A, chow_patel_tag()) (Chow-Patel parallel ILU0)."""
    _create = "vclgbChowPatelIluCreate"


class chow_patel_icc_precond(_ChowPatel):
    """chow_patel_icc_precond<compressed_matrix>(A, chow_patel_tag()) (Chow-Patel parallel IC0)."""
    _create = "vclgbChowPatelIccCreate"


def solve(A, b, tag, precond=None, x=None):
    """linalg::solve(A, b, tag[, precond]) -> x (device tensor).

    Raises on failures other than NOT_CONVERGED/BREAKDOWN, which the reference
    reports only through tag.iters()/tag.error(); those are in tag.status()."""
    torch = _torch()
    dt = A.dtype
    b = b if (isinstance(b, torch.Tensor) and b.is_cuda and b.dtype == dt) else _dev(b, dt)
    if x is None:
        x = torch.empty(A.size1(), dtype=dt, device="cuda")
    be, lib = A.be, A.be.lib
    t = ctypes.byref(tag.t)
    ok = (NOT_CONVERGED, BREAKDOWN)
    if isinstance(tag, refined_cg_tag):
        outer = _U32()
        be.check(lib.vclgbSolveRefinedCG(be.h, A.h, _ptr(b), _ptr(x), t, tag.inner_tol,
                                         tag.max_outer, ctypes.byref(outer)), ok)
        tag.outer = outer.value
    elif isinstance(tag, mixed_precision_cg_tag):
        be.check(lib.vclgbSolveMixedCG(be.h, A.h, _ptr(b), _ptr(x), t, tag.inner_tol), ok)
    elif isinstance(tag, cg_tag):
        be.check(lib.vclgbSolveCG(be.h, A.h, _ptr(b), _ptr(x), t,
                                  precond.h if precond else _P(0)), ok)
    elif isinstance(tag, bicgstab_tag):
        be.check(lib.vclgbSolveBiCGStab(be.h, A.h, _ptr(b), _ptr(x), t,
                                        precond.h if precond else _P(0)), ok)
    elif isinstance(tag, gmres_tag):
        be.check(lib.vclgbSolveGMRES(be.h, A.h, _ptr(b), _ptr(x), t,
                                     precond.h if precond else _P(0)), ok)
    else:
        raise TypeError("unknown solver tag")
    return x


# ---- batched solves (no reference counterpart) ---------------------------------
class Batch:
    """Independent systems = diagonal blocks of one block-diagonal CSR matrix.
    methods[k]: 0 = pipelined CG, 1 = pipelined BiCGStab."""

    def __init__(self, A, sys_ptr, methods):
        self.be = A.be
        self._A = A
        self.sys_ptr = np.ascontiguousarray(sys_ptr, dtype=np.uint32)
        self.methods = np.ascontiguousarray(methods, dtype=np.int32)
        self.nsys = len(self.methods)
        h = _P()
        self.be.check(self.be.lib.vclgbBatchCreate(
            self.be.h, A.h, self.nsys, self.sys_ptr.ctypes.data_as(_P),
            self.methods.ctypes.data_as(_P), ctypes.byref(h)))
        self.h = h

    def tune(self, b):
        blk, ln = ctypes.c_int32(), ctypes.c_int32()
        self.be.check(self.be.lib.vclgbBatchTune(self.be.h, self.h, _ptr(b), ctypes.byref(blk),
                                                 ctypes.byref(ln)))
        return blk.value, ln.value

    def solve(self, b, tol=1e-10, max_iters=10000, x=None):
        torch = _torch()
        b = b if (isinstance(b, torch.Tensor) and b.is_cuda) else _dev(b, torch.float64)
        if x is None:
            x = torch.empty_like(b)
        it = np.zeros(self.nsys, np.uint32)
        st = np.zeros(self.nsys, np.int32)
        er = np.zeros(self.nsys, np.float64)
        self.be.check(self.be.lib.vclgbBatchSolve(self.be.h, self.h, _ptr(b), _ptr(x), float(tol),
                                                  int(max_iters), it.ctypes.data_as(_P),
                                                  st.ctypes.data_as(_P), er.ctypes.data_as(_P)),
                      (NOT_CONVERGED,))
        return x, it, st, er

    def __del__(self):
        if _exiting:
            return
        try:
            if self.h:
                self.be.lib.vclgbBatchDestroy(ctypes.byref(self.h))
        except Exception:
            pass


# ---- adjoint (backward) solve ---------------------------------------------------
_SOLVER_IDS = {"cg": 0, "bicgstab": 1, "gmres": 2}


def solve_adjoint(A, x, dLdx, tag, solver="cg", precond=None, symmetric=False, want_dA=True):
    """Backward of x = A^-1 b: returns (dL/db, dL/dA on A's pattern or None)."""
    torch = _torch()
    dt = A.dtype
    x = x if (isinstance(x, torch.Tensor) and x.is_cuda) else _dev(x, dt)
    dLdx = dLdx if (isinstance(dLdx, torch.Tensor) and dLdx.is_cuda) else _dev(dLdx, dt)
    lam = torch.empty(A.size1(), dtype=dt, device="cuda")
    gA = torch.empty(max(A.nnz(), 1), dtype=dt, device="cuda") if want_dA else None
    A.be.check(A.be.lib.vclgbSolveAdjoint(A.be.h, A.h, _SOLVER_IDS[solver],
                                          precond.h if precond else _P(0), _ptr(x), _ptr(dLdx),
                                          _ptr(lam), _ptr(gA) if want_dA else _P(0),
                                          ctypes.byref(tag.t), 1 if symmetric else 0),
               (NOT_CONVERGED, BREAKDOWN))
    return lam, (gA[:A.nnz()] if want_dA else None)


def transpose_export(A, which, count, dtype):
    torch = _torch()
    out = torch.empty(max(int(count), 1), dtype=dtype, device="cuda")
    A.be.check(A.be.lib.vclgbTransposeExport(A.be.h, A.h, which, _ptr(out)))
    return out[:int(count)]
