"""Seeded synthetic sparse systems (numpy, PCG64 via default_rng).

Every generator returns CSR arrays (row_ptr uint32, cols uint32 sorted within
rows, values float64) so the same arrays feed the GPU engine and the CPU
oracle.  Sizes follow the workloads the engine is measured on:

  laplace2d(256, 256)        2D 5-point Dirichlet Laplacian (tools/matrix_generation.hpp:47-87
                             ordering: row = i + j*nx, 4 on the diagonal, -1 off it)
  laplace3d(128)             3D 7-point Laplacian, 2,097,152 rows
  lognormal_random(n, ...)   random nonsymmetric rows, lengths lognormal(2.5, 1) clipped to
                             [1, 2000], distinct uniform columns, N(0,1) values, diagonal
                             shifted by 1.1 x the row's absolute sum
  diffusion3d(192, ...)      cell-centred variable-coefficient diffusion, kappa = exp(g) for a
                             Gaussian random field g (correlation length 8 cells) scaled to a
                             max/min contrast of 1e4, harmonic-mean face coefficients
  diffusion2d_edges(512,...) 2D diffusion with per-edge log-normal coefficients
  convdiff2d(nx, ny, pe)     first-order upwind convection-diffusion (nonsymmetric)
"""
import numpy as np


def _stencil_csr(shape, offsets, weights):
    """CSR of a constant-coefficient stencil on a grid (Dirichlet: neighbours
    outside the grid dropped).  offsets: list of per-axis offset tuples in
    increasing order of the flat column offset; weights: matching values."""
    dims = len(shape)
    n = int(np.prod(shape))
    idx = np.indices(shape[::-1]).reshape(dims, -1)[::-1]  # idx[0] fastest axis
    valid = []
    for off in offsets:
        m = np.ones(n, dtype=bool)
        for ax, o in enumerate(off):
            if o < 0:
                m &= idx[ax] >= -o
            elif o > 0:
                m &= idx[ax] < shape[ax] - o
        valid.append(m)
    valid = np.stack(valid)                       # (k, n)
    counts = valid.sum(axis=0).astype(np.int64)
    rp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=rp[1:])
    nnz = int(rp[-1])
    cols = np.empty(nnz, dtype=np.uint32)
    vals = np.empty(nnz, dtype=np.float64)
    pos = rp[:-1].copy()
    strides = [1]
    for s in shape[:-1]:
        strides.append(strides[-1] * s)
    rows = np.arange(n, dtype=np.int64)
    for k, off in enumerate(offsets):
        m = valid[k]
        flat = sum(o * st for o, st in zip(off, strides))
        r = rows[m]
        p = pos[m]
        cols[p] = (r + flat).astype(np.uint32)
        w = weights[k]
        vals[p] = w[m] if isinstance(w, np.ndarray) else w
        pos[m] += 1
    return rp.astype(np.uint32), cols, vals


def laplace2d(nx, ny=None, scaled=False):
    ny = nx if ny is None else ny
    offs = [(0, -1), (-1, 0), (0, 0), (1, 0), (0, 1)]
    w = [-1.0, -1.0, 4.0, -1.0, -1.0]
    rp, ci, v = _stencil_csr((nx, ny), offs, w)
    if scaled:  # h = 1/(nx+1): scales x, not the iteration count
        v = v * float((nx + 1) ** 2)
    return rp, ci, v


def laplace3d(n):
    offs = [(0, 0, -1), (0, -1, 0), (-1, 0, 0), (0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)]
    w = [-1.0, -1.0, -1.0, 6.0, -1.0, -1.0, -1.0]
    return _stencil_csr((n, n, n), offs, w)


def lognormal_random(n, mu=2.5, sigma=1.0, lo=1, hi=2000, seed=1):
    """Random nonsymmetric matrix with lognormal row lengths (diagonal included)."""
    rng = np.random.default_rng(seed)
    L = np.clip(np.rint(rng.lognormal(mu, sigma, n)), lo, min(hi, n)).astype(np.int64)
    off = L - 1
    rows = np.repeat(np.arange(n, dtype=np.int64), off)
    c = rng.integers(0, n - 1, size=rows.size, dtype=np.int64)
    c += (c >= rows)  # skip the diagonal
    def sorted_unique(k):
        k.sort()
        keep = np.empty(k.size, dtype=bool)
        keep[:1] = True
        np.not_equal(k[1:], k[:-1], out=keep[1:])
        return k[keep]

    keys = sorted_unique(rows * n + c)
    for _ in range(64):  # redraw the (rare) repeated columns
        cnt = np.bincount(keys // n, minlength=n)
        deficit = off - cnt
        if not deficit.any():
            break
        rr = np.repeat(np.nonzero(deficit)[0].astype(np.int64), deficit[deficit > 0])
        cc = rng.integers(0, n - 1, size=rr.size, dtype=np.int64)
        cc += (cc >= rr)
        keys = sorted_unique(np.concatenate([keys, rr * n + cc]))
    # add the diagonal and sort (row, col)
    diag = np.arange(n, dtype=np.int64) * (n + 1)
    keys = np.concatenate([keys, diag])
    keys.sort()
    rows = keys // n
    cols = (keys - rows * n).astype(np.uint32)
    vals = rng.standard_normal(keys.size)
    rowsum = np.bincount(rows, weights=np.abs(vals), minlength=n)
    isdiag = cols.astype(np.int64) == rows
    vals[isdiag] += 1.1 * rowsum
    rp = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n), out=rp[1:])
    return rp.astype(np.uint32), cols, vals


def gaussian_field(shape, corr, rng):
    """Zero-mean unit-variance Gaussian random field with a Gaussian covariance
    of correlation length `corr` cells (white noise filtered in Fourier space)."""
    noise = rng.standard_normal(shape)
    F = np.fft.rfftn(noise)
    ks = [np.fft.fftfreq(s) for s in shape[:-1]] + [np.fft.rfftfreq(shape[-1])]
    grids = np.meshgrid(*ks, indexing="ij", sparse=True)
    k2 = sum(g * g for g in grids)
    F *= np.exp(-2.0 * (np.pi ** 2) * (corr ** 2) * k2)
    g = np.fft.irfftn(F, s=shape, axes=tuple(range(len(shape))))
    g -= g.mean()
    g /= g.std()
    return g


def _fv_diffusion(kap, face_k):
    """Assemble a cell-centred diffusion matrix given per-axis face coefficients
    face_k[ax] (arrays of shape with that axis one shorter) and boundary cells'
    kappa for Dirichlet faces (coefficient 2*kappa)."""
    shape = kap.shape
    dims = len(shape)
    n = kap.size
    diag = np.zeros(shape)
    offs, weights = [], []
    # flat ordering: axis 0 fastest (row = i + nx*(j + ny*k)), arrays indexed [i, j, k]
    for ax in range(dims):
        fk = face_k[ax]
        lo = [slice(None)] * dims
        hi = [slice(None)] * dims
        lo[ax] = slice(0, shape[ax] - 1)
        hi[ax] = slice(1, shape[ax])
        diag[tuple(lo)] += fk
        diag[tuple(hi)] += fk
        # Dirichlet boundary faces
        b0 = [slice(None)] * dims
        b1 = [slice(None)] * dims
        b0[ax] = 0
        b1[ax] = shape[ax] - 1
        diag[tuple(b0)] += 2.0 * kap[tuple(b0)]
        diag[tuple(b1)] += 2.0 * kap[tuple(b1)]
        wm = np.zeros(shape)   # coupling to the lower neighbour along ax
        wp = np.zeros(shape)   # coupling to the upper neighbour
        wm[tuple(hi)] = -fk
        wp[tuple(lo)] = -fk
        om = [0] * dims
        op = [0] * dims
        om[ax] = -1
        op[ax] = 1
        offs += [tuple(om), tuple(op)]
        weights += [wm, wp]
    offs.append(tuple([0] * dims))
    weights.append(diag)
    # sort offsets by flat column offset (axis 0 fastest)
    strides = [1]
    for s in shape[:-1]:
        strides.append(strides[-1] * s)
    flat = [sum(o * st for o, st in zip(off, strides)) for off in offs]
    order = np.argsort(flat)
    offs = [offs[i] for i in order]
    # weights as flat arrays in row order (axis 0 fastest => Fortran order)
    wflat = [weights[i].reshape(-1, order="F") for i in order]
    return _stencil_csr(shape, offs, wflat)


def diffusion3d(N=192, corr=8.0, contrast=1e4, seed=2):
    """Variable-coefficient 3D diffusion; returns (rp, ci, v, f)."""
    rng = np.random.default_rng(seed)
    g = gaussian_field((N, N, N), corr, rng)
    a = np.log(contrast) / (g.max() - g.min())
    kap = np.exp(a * (g - g.min()))
    faces = []
    for ax in range(3):
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[ax] = slice(0, N - 1)
        hi[ax] = slice(1, N)
        k1, k2 = kap[tuple(lo)], kap[tuple(hi)]
        faces.append(2.0 * k1 * k2 / (k1 + k2))
    rp, ci, v = _fv_diffusion(kap, faces)
    f = rng.uniform(0.0, 1.0, N ** 3)
    return rp, ci, v, f


def diffusion2d_edges(N=512, contrast=1e3, seed=4):
    """2D diffusion with per-edge log-normal coefficients; returns (rp, ci, v, edge_k)
    where edge_k = (kx [N-1, N], ky [N, N-1]) are the face coefficients."""
    rng = np.random.default_rng(seed)
    zx = rng.standard_normal((N - 1, N))
    zy = rng.standard_normal((N, N - 1))
    zmin = min(zx.min(), zy.min())
    zmax = max(zx.max(), zy.max())
    a = np.log(contrast) / (zmax - zmin)
    kx = np.exp(a * (zx - zmin))
    ky = np.exp(a * (zy - zmin))
    kap = np.ones((N, N))
    rp, ci, v = _fv_diffusion(kap, [kx, ky])
    return rp, ci, v, (kx, ky)


def convdiff2d(nx, ny=None, peclet=10.0, shift=0.0):
    """Upwind convection-diffusion -lap(u) + pe*(u_x + u_y) on a unit grid
    (flow in +x and +y), scaled by h^2: nonsymmetric M-matrix."""
    ny = nx if ny is None else ny
    h = 1.0 / (max(nx, ny) + 1)
    c = peclet * h  # upwind convection coefficient after scaling by h^2
    offs = [(0, -1), (-1, 0), (0, 0), (1, 0), (0, 1)]
    w = [-1.0 - c, -1.0 - c, 4.0 + 2.0 * c + shift, -1.0, -1.0]
    return _stencil_csr((nx, ny), offs, w)


def rhs_uniform(n, seed, lo=-1.0, hi=1.0):
    return np.random.default_rng(seed).uniform(lo, hi, n)


def batch_systems(count=4096, lo=500, hi=20000, seed=3):
    """Independent systems for the batched solver, as one block-diagonal CSR.

    Sizes n_k are drawn log-uniform in [lo, hi] and rounded to a near-square
    grid nx*ny.  Even k: SPD 2D 5-point Laplacian plus a diagonal shift
    U[0.01, 1] (solved with CG); odd k: nonsymmetric upwind convection-diffusion
    with Peclet number U[0.1, 50] (solved with BiCGStab).  Returns
    (rp, ci, v, sys_ptr, methods, b) with b ~ U[-1, 1]."""
    rng = np.random.default_rng(seed)
    target = np.exp(rng.uniform(np.log(lo), np.log(hi), count))
    shifts = rng.uniform(0.01, 1.0, count)
    pecl = rng.uniform(0.1, 50.0, count)
    rps, cis, vs, sizes, methods = [], [], [], [], []
    row0 = 0
    nnz0 = 0
    for k in range(count):
        nx = max(2, int(round(np.sqrt(target[k]))))
        ny = max(2, int(round(target[k] / nx)))
        if k % 2 == 0:
            rp, ci, v = laplace2d(nx, ny)
            v = v.copy()
            v[ci.astype(np.int64) == np.repeat(np.arange(nx * ny), np.diff(rp.astype(np.int64)))] += shifts[k]
            methods.append(0)
        else:
            rp, ci, v = convdiff2d(nx, ny, peclet=pecl[k])
            methods.append(1)
        n = nx * ny
        rps.append(rp[:-1].astype(np.int64) + nnz0)
        cis.append(ci.astype(np.int64) + row0)
        vs.append(v)
        sizes.append(n)
        row0 += n
        nnz0 += int(rp[-1])
    rp = np.concatenate(rps + [np.array([nnz0])]).astype(np.uint32)
    ci = np.concatenate(cis).astype(np.uint32)
    v = np.concatenate(vs)
    sys_ptr = np.zeros(count + 1, np.uint32)
    sys_ptr[1:] = np.cumsum(sizes)
    b = rng.uniform(-1.0, 1.0, row0)
    return rp, ci, v, sys_ptr, np.array(methods, np.int32), b
