"""Synthetic sparse systems with the shapes used by the spaND benchmarks.

The reference ships −Δ fixtures as Matrix Market files (``mats/neglapl_{d}_{n}.mm``:
2d on the diagonal, −1 off the diagonal, row-major grid numbering, Dirichlet) and builds
grid coordinates with ``linspace_nd`` (``src/util.cpp:488-517``: coordinate 0 is the
slowest grid index).  These generators reproduce both bit for bit and add the other
workloads (high-contrast finite-volume diffusion, reaction-diffusion batches, anisotropic
diffusion with per-face conductivities).  All matrices are returned as CSC with sorted
int32 row indices and no duplicate entries.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def _canonical(A: sp.spmatrix) -> sp.csc_matrix:
    A = sp.csc_matrix(A)
    A.sum_duplicates()
    A.sort_indices()
    A.indices = A.indices.astype(np.int32)
    A.indptr = A.indptr.astype(np.int32)
    return A


def linspace_nd(n: int, dim: int) -> np.ndarray:
    """Grid coordinates, shape (dim, n**dim); coordinate 0 varies slowest (util.cpp:488-517)."""
    axes = np.meshgrid(*([np.arange(n, dtype=np.float64)] * dim), indexing="ij")
    return np.stack([a.reshape(-1) for a in axes], axis=0)


def neglapl(n: int, dim: int) -> sp.csc_matrix:
    """−Δ on an n^dim grid, 2·dim on the diagonal, −1 to each grid neighbour (mats/neglapl_*.mm)."""
    N = n ** dim
    idx = np.arange(N).reshape((n,) * dim)
    rows, cols = [np.arange(N)], [np.arange(N)]
    vals = [np.full(N, 2.0 * dim)]
    for ax in range(dim):
        a = np.take(idx, np.arange(n - 1), axis=ax).reshape(-1)
        b = np.take(idx, np.arange(1, n), axis=ax).reshape(-1)
        rows += [a, b]
        cols += [b, a]
        vals += [np.full(a.size, -1.0), np.full(a.size, -1.0)]
    A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    return _canonical(A)


def neglapl_unsym(n: int, dim: int, seed: int = 0, amp: float = 0.1) -> sp.csc_matrix:
    """−Δ plus U(−amp, amp) on every stored entry: a nonsymmetric matrix with the Laplacian's
    pattern, as the reference's tests build their GEN problems (tests/tests.cpp:98-109;
    there with std::default_random_engine, here with numpy's generator from `seed`)."""
    A = neglapl(n, dim).copy()
    A.data += np.random.default_rng(seed).uniform(-amp, amp, A.nnz)
    return A


def face_diffusion(n: int, dim: int, face_k: list[np.ndarray], shift: np.ndarray | None = None) -> sp.csc_matrix:
    """Finite-volume diffusion with conductivity face_k[ax][face] on the faces between
    grid neighbours along axis ax (Dirichlet: a boundary face has the conductivity of its
    cell's interior neighbour face, i.e. the same weight as a −Δ boundary row), plus an
    optional diagonal shift.  face_k[ax] has shape (n-1,) along ax times n on the others."""
    N = n ** dim
    idx = np.arange(N).reshape((n,) * dim)
    diag = np.zeros((n,) * dim)
    rows, cols, vals = [], [], []
    for ax in range(dim):
        kf = np.asarray(face_k[ax], dtype=np.float64)
        a = np.take(idx, np.arange(n - 1), axis=ax).reshape(-1)
        b = np.take(idx, np.arange(1, n), axis=ax).reshape(-1)
        w = kf.reshape(-1)
        rows += [a, b]
        cols += [b, a]
        vals += [-w, -w]
        d = np.zeros((n,) * dim)
        sl_lo = [slice(None)] * dim
        sl_hi = [slice(None)] * dim
        sl_lo[ax] = slice(0, n - 1)
        sl_hi[ax] = slice(1, n)
        d[tuple(sl_lo)] += kf
        d[tuple(sl_hi)] += kf
        # Dirichlet boundary faces carry the conductivity of the adjacent interior face
        first = [slice(None)] * dim
        last = [slice(None)] * dim
        first[ax] = slice(0, 1)
        last[ax] = slice(n - 1, n)
        kf0 = np.take(kf, [0], axis=ax)
        kf1 = np.take(kf, [n - 2], axis=ax)
        d[tuple(first)] += kf0
        d[tuple(last)] += kf1
        diag += d
    dg = diag.reshape(-1)
    if shift is not None:
        dg = dg + np.asarray(shift, dtype=np.float64).reshape(-1)
    rows.append(np.arange(N))
    cols.append(np.arange(N))
    vals.append(dg)
    A = sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    return _canonical(A)


def face_diffusion_map(n: int, dim: int):
    """The linear map from face conductivities to the CSC values of face_diffusion(n, dim, ·):
    with w the axis-by-axis concatenation of the flattened (C order) face arrays,
    values = zeros(nnz); values[pos[t]] += coef[t] * w[face[t]] for every t.  Returns
    (pattern, pos, face, coef), pattern being the CSC matrix for unit conductivities."""
    N = n ** dim
    idx = np.arange(N).reshape((n,) * dim)
    rows, cols, face, coef = [], [], [], []
    base = 0
    for ax in range(dim):
        shape = [n] * dim
        shape[ax] = n - 1
        fid = base + np.arange(int(np.prod(shape))).reshape(shape)
        a = np.take(idx, np.arange(n - 1), axis=ax).reshape(-1)
        b = np.take(idx, np.arange(1, n), axis=ax).reshape(-1)
        f = fid.reshape(-1)
        for r, c, k in ((a, b, -1.0), (b, a, -1.0), (a, a, 1.0), (b, b, 1.0)):
            rows.append(r)
            cols.append(c)
            face.append(f)
            coef.append(np.full(f.size, k))
        # Dirichlet boundary cells: the conductivity of their interior neighbour face
        for layer, fl in ((0, 0), (n - 1, n - 2)):
            cell = np.take(idx, [layer], axis=ax).reshape(-1)
            rows.append(cell)
            cols.append(cell)
            face.append(np.take(fid, [fl], axis=ax).reshape(-1))
            coef.append(np.ones(cell.size))
        base += fid.size
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    face, coef = np.concatenate(face), np.concatenate(coef)
    pattern = _canonical(sp.coo_matrix((np.ones(rows.size), (rows, cols)), shape=(N, N)))
    # CSC position of every (row, col): CSC order is (col, row) lexicographic
    pcol = np.repeat(np.arange(N, dtype=np.int64), np.diff(pattern.indptr))
    keys = pcol * N + pattern.indices.astype(np.int64)
    pos = np.searchsorted(keys, cols.astype(np.int64) * N + rows)
    return pattern, pos, face, coef


def high_contrast_fv2d(n: int = 1024, tile: int = 8, seed: int = 0) -> sp.csc_matrix:
    """2D 5-point finite-volume diffusion, cell coefficients 10^U(−3,3) constant on
    tile×tile blocks, harmonic-mean face conductivities, Dirichlet."""
    rng = np.random.default_rng(seed)
    nt = (n + tile - 1) // tile
    kt = 10.0 ** rng.uniform(-3.0, 3.0, size=(nt, nt))
    kc = np.repeat(np.repeat(kt, tile, axis=0), tile, axis=1)[:n, :n]
    f0 = 2.0 * kc[:-1, :] * kc[1:, :] / (kc[:-1, :] + kc[1:, :])
    f1 = 2.0 * kc[:, :-1] * kc[:, 1:] / (kc[:, :-1] + kc[:, 1:])
    return face_diffusion(n, 2, [f0, f1])


def reaction_diffusion3d(n: int, c: float) -> sp.csc_matrix:
    """−Δ + c·I on an n³ grid (7-point)."""
    A = neglapl(n, 3)
    return _canonical(A + c * sp.identity(A.shape[0], format="csc"))


def anisotropic3d(n: int, theta: list[np.ndarray], scaling=(1.0, 1.0, 0.01)) -> sp.csc_matrix:
    """3D 7-point diffusion with per-face conductivities scaling[ax]·theta[ax]."""
    return face_diffusion(n, 3, [scaling[ax] * np.asarray(theta[ax]) for ax in range(3)])


def anisotropic_theta(n: int, seed: int = 0) -> list[np.ndarray]:
    """Per-face conductivities θ = exp(0.5·z), z ~ N(0,1)."""
    rng = np.random.default_rng(seed)
    shapes = []
    for ax in range(3):
        s = [n, n, n]
        s[ax] = n - 1
        shapes.append(tuple(s))
    return [np.exp(0.5 * rng.standard_normal(s)) for s in shapes]


def rhs(n: int, nrhs: int = 1, seed: int = 0) -> np.ndarray:
    """Right-hand sides ~ N(0,1), column-major (n, nrhs)."""
    rng = np.random.default_rng(seed)
    b = rng.standard_normal((nrhs, n)).T
    return np.asfortranarray(b)
