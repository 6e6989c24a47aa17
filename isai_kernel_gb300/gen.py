"""Seeded synthetic BSR systems for the block-ILU(0) + ISAI path.

The reference runs on external Matrix Market files that are not part of it;
these generators stand in for them with the shapes, sizes and value
distributions of the five workloads the preconditioner is measured on:

* ``laplace2d``      2D 5-point, 4 coupled DOF per node (4x4 blocks):
                     diagonal block 4*I + R, neighbour blocks -I + R, R with
                     zero diagonal and off-diagonal entries U[-c, c].
* ``convdiff3d``     3D 7-point upwinded convection-diffusion, velocity
                     (1, 0.5, 0.25), cell Peclet 10 along the fastest axis,
                     stencil (x) I_4 plus couplings U[-0.05, 0.05].
* ``powerlaw``       random unsymmetric block matrix, 8x8 blocks, power-law
                     off-diagonal block counts per row (alpha 2.1, rescaled to
                     mean 12, max 2000), uniform columns, row-sum dominance 1.2.
* ``lognormal2d``    2D 5-point diffusion with a log-normal coefficient field
                     (Gaussian random field, sigma 1, correlation length 16).
* ``batch_laplace2d`` many ``laplace2d`` systems with random grid sides.

All randomness comes from ``numpy.random.default_rng(seed)`` (PCG64), drawn in
BSR order, so a seed fixes the matrix bit for bit on every host.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class BSRMatrix:
    """Block sparse row matrix: 0-based int32 ``rowptr[nb+1]``, ``colind[nnzb]``
    ascending per row, ``val[nnzb, bs, bs]`` row-major blocks (float64)."""

    nb: int
    bs: int
    rowptr: np.ndarray
    colind: np.ndarray
    val: np.ndarray

    @property
    def nnzb(self) -> int:
        return int(self.colind.shape[0])

    @property
    def n(self) -> int:
        return self.nb * self.bs

    def copy(self) -> "BSRMatrix":
        return BSRMatrix(self.nb, self.bs, self.rowptr.copy(), self.colind.copy(), self.val.copy())

    def to_dense(self) -> np.ndarray:
        n, bs = self.n, self.bs
        D = np.zeros((n, n))
        for i in range(self.nb):
            for p in range(self.rowptr[i], self.rowptr[i + 1]):
                j = self.colind[p]
                D[i * bs:(i + 1) * bs, j * bs:(j + 1) * bs] = self.val[p]
        return D

    def to_csr(self):
        """Scalar CSR (row direction): returns (rowptr, colind, val)."""
        bs = self.bs
        lens = np.diff(self.rowptr).astype(np.int64) * bs
        row_len = np.repeat(lens, bs)
        rp = np.zeros(self.n + 1, dtype=np.int64)
        np.cumsum(row_len, out=rp[1:])
        cols, vals = [], []
        for i in range(self.nb):
            s, e = self.rowptr[i], self.rowptr[i + 1]
            c = (self.colind[s:e, None] * bs + np.arange(bs)[None, :]).reshape(-1)
            for r in range(bs):
                cols.append(c)
                vals.append(self.val[s:e, r, :].reshape(-1))
        col = np.concatenate(cols) if cols else np.zeros(0, np.int64)
        val = np.concatenate(vals) if vals else np.zeros(0)
        return rp.astype(np.int32), col.astype(np.int32), val.astype(np.float64)


def _assemble(nb: int, bs: int, cols: np.ndarray, coef: np.ndarray) -> tuple:
    """cols/coef: (nb, k) arrays with -1 marking absent entries, columns
    ascending along axis 1.  Returns rowptr, colind, per-block scalar coef."""
    mask = cols >= 0
    counts = mask.sum(axis=1)
    rowptr = np.zeros(nb + 1, dtype=np.int32)
    np.cumsum(counts, out=rowptr[1:])
    return rowptr, cols[mask].astype(np.int32), coef[mask]


def _blocks(scal: np.ndarray, bs: int, rng, coupling: float, diag_zero: bool = True,
            relative: bool = False) -> np.ndarray:
    nnzb = scal.shape[0]
    R = rng.uniform(-coupling, coupling, size=(nnzb, bs, bs))
    if diag_zero:
        idx = np.arange(bs)
        R[:, idx, idx] = 0.0
    if relative:
        R *= np.abs(scal)[:, None, None]
    val = R
    idx = np.arange(bs)
    val[:, idx, idx] += scal[:, None]
    return val


def laplace2d(side: int, bs: int = 4, seed: int = 0, coupling: float = 0.1) -> BSRMatrix:
    """2D 5-point Laplacian on a side x side grid (node = y*side + x)."""
    nb = side * side
    node = np.arange(nb)
    x, y = node % side, node // side
    offs = [(-side, y > 0), (-1, x > 0), (0, np.ones(nb, bool)), (1, x < side - 1),
            (side, y < side - 1)]
    cols = np.stack([np.where(m, node + o, -1) for o, m in offs], axis=1)
    coef = np.stack([np.full(nb, 4.0 if o == 0 else -1.0) for o, _ in offs], axis=1)
    rowptr, colind, scal = _assemble(nb, bs, cols, coef)
    rng = np.random.default_rng(seed)
    return BSRMatrix(nb, bs, rowptr, colind, _blocks(scal, bs, rng, coupling))


def convdiff3d(side: int, bs: int = 4, seed: int = 0, velocity=(1.0, 0.5, 0.25),
               peclet: float = 10.0, coupling: float = 0.05) -> BSRMatrix:
    """3D 7-point upwinded convection-diffusion, Dirichlet boundary, scaled by
    h^2/nu (node = (z*side + y)*side + x).  Pe_d = peclet * v_d / max|v|."""
    nb = side ** 3
    node = np.arange(nb, dtype=np.int64)
    x, y, z = node % side, (node // side) % side, node // (side * side)
    vmax = max(abs(v) for v in velocity)
    pe = [peclet * v / vmax for v in velocity]
    # first-order upwind for positive velocities: backward neighbour gets -(1+Pe)
    s2 = side * side
    offs = [(-s2, z > 0, -(1 + pe[2])), (-side, y > 0, -(1 + pe[1])),
            (-1, x > 0, -(1 + pe[0])), (0, None, 6.0 + sum(pe)), (1, x < side - 1, -1.0),
            (side, y < side - 1, -1.0), (s2, z < side - 1, -1.0)]
    cols = np.stack([node + o if m is None else np.where(m, node + o, -1) for o, m, _ in offs],
                    axis=1)
    coef = np.stack([np.full(nb, c) for _, _, c in offs], axis=1)
    rowptr, colind, scal = _assemble(nb, bs, cols, coef)
    rng = np.random.default_rng(seed)
    return BSRMatrix(nb, bs, rowptr, colind, _blocks(scal, bs, rng, coupling))


def powerlaw(nb: int, bs: int = 8, seed: int = 0, alpha: float = 2.1, mean: float = 12.0,
             kmax: int = 2000, dominance: float = 1.2) -> BSRMatrix:
    """Random unsymmetric block matrix with power-law off-diagonal block
    counts per row (discrete P(k) ~ k^-alpha on [1, kmax], scaled by
    mean/E[k], rounded, clipped to [1, min(kmax, nb-1)]), columns uniform
    without the diagonal (duplicates dropped), off-diagonal entries U[-1,1],
    and the diagonal entry of every scalar row set to dominance * sum|off|."""
    rng = np.random.default_rng(seed)
    k = np.arange(1, kmax + 1, dtype=np.float64)
    p = k ** (-alpha)
    p /= p.sum()
    raw = rng.choice(np.arange(1, kmax + 1), size=nb, p=p)
    cnt = np.clip(np.rint(raw * (mean / float((k * p).sum()))), 1, min(kmax, max(nb - 1, 1)))
    cnt = cnt.astype(np.int64) if nb > 1 else np.zeros(nb, np.int64)
    rows = np.repeat(np.arange(nb, dtype=np.int64), cnt)
    c = rng.integers(0, max(nb - 1, 1), size=rows.shape[0], dtype=np.int64)
    c = c + (c >= rows)  # skip the diagonal
    rows = np.concatenate([rows, np.arange(nb, dtype=np.int64)])
    c = np.concatenate([c, np.arange(nb, dtype=np.int64)])
    key = np.unique(rows * nb + c)
    rows, c = key // nb, key % nb
    rowptr = np.zeros(nb + 1, dtype=np.int32)
    np.cumsum(np.bincount(rows, minlength=nb), out=rowptr[1:])
    colind = c.astype(np.int32)
    val = rng.uniform(-1.0, 1.0, size=(colind.shape[0], bs, bs))
    is_diag = rows == c
    dpos = np.nonzero(is_diag)[0]
    absrow = np.zeros((nb, bs))
    np.add.at(absrow, rows, np.abs(val).sum(axis=2))
    idx = np.arange(bs)
    absrow -= np.abs(val[dpos][:, idx, idx])
    val[dpos[:, None], idx[None, :], idx[None, :]] = dominance * absrow
    return BSRMatrix(nb, bs, rowptr, colind, val)


def gaussian_field(side: int, seed: int, sigma: float = 1.0, corr_len: float = 16.0) -> np.ndarray:
    """Stationary Gaussian random field on a periodic side x side grid:
    white noise filtered in Fourier space by exp(-(k*corr_len)^2/4)
    (squared-exponential covariance of length corr_len), normalised to
    standard deviation sigma."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((side, side))
    kx = np.fft.fftfreq(side) * 2 * np.pi
    K2 = kx[:, None] ** 2 + kx[None, :] ** 2
    f = np.real(np.fft.ifft2(np.fft.fft2(w) * np.exp(-K2 * corr_len ** 2 / 4.0)))
    f -= f.mean()
    sd = f.std()
    return sigma * f / (sd if sd > 0 else 1.0)


def lognormal2d(side: int, bs: int = 4, seed: int = 0, sigma: float = 1.0,
                corr_len: float = 16.0, coupling: float = 0.05) -> BSRMatrix:
    """2D 5-point diffusion -div(kappa grad u), kappa = exp(G), harmonic-mean
    face coefficients, Dirichlet boundary; blocks coef*I + relative couplings
    U[-coupling, coupling]*|coef|."""
    kap = np.exp(gaussian_field(side, seed, sigma, corr_len)).reshape(-1)
    nb = side * side
    node = np.arange(nb)
    x, y = node % side, node // side

    def face(o, m):
        nbr = np.where(m, node + o, node)
        return np.where(m, 2 * kap * kap[nbr] / (kap + kap[nbr]), kap)

    fs = face(-side, y > 0)
    fw = face(-1, x > 0)
    fe = face(1, x < side - 1)
    fn = face(side, y < side - 1)
    diag = fs + fw + fe + fn
    offs = [(-side, y > 0, -fs), (-1, x > 0, -fw), (0, np.ones(nb, bool), diag),
            (1, x < side - 1, -fe), (side, y < side - 1, -fn)]
    cols = np.stack([np.where(m, node + o, -1) for o, m, _ in offs], axis=1)
    coef = np.stack([c for _, _, c in offs], axis=1)
    rowptr, colind, scal = _assemble(nb, bs, cols, coef)
    rng = np.random.default_rng(seed + 1)
    return BSRMatrix(nb, bs, rowptr, colind,
                     _blocks(scal, bs, rng, coupling, relative=True))


def rhs(n: int, seed: int = 0, k: int = 1) -> np.ndarray:
    """Uniform [-1, 1] right-hand side(s): shape (n,) or (n, k) column-major
    semantics (column c drawn after column c-1)."""
    rng = np.random.default_rng(seed)
    if k == 1:
        return rng.uniform(-1.0, 1.0, size=n)
    return np.ascontiguousarray(rng.uniform(-1.0, 1.0, size=(k, n)).T)


def batch_laplace2d(count: int = 256, side_lo: int = 32, side_hi: int = 512, bs: int = 4,
                    seed: int = 0, nrhs: int = 32):
    """``count`` independent ``laplace2d`` systems, grid side ~ U{side_lo..side_hi}
    (system s uses seed+s), each with ``nrhs`` uniform right-hand sides."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(side_lo, side_hi + 1, size=count)
    out = []
    for s, side in enumerate(sides):
        A = laplace2d(int(side), bs=bs, seed=seed + s)
        out.append((A, rhs(A.n, seed=seed + s, k=nrhs)))
    return out


def write_mtx(path: str, A: BSRMatrix) -> None:
    """Matrix Market coordinate real general, 1-based, every stored entry."""
    rp, ci, v = A.to_csr()
    rows = np.repeat(np.arange(A.n), np.diff(rp))
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate real general\n")
        f.write(f"{A.n} {A.n} {len(v)}\n")
        for r, c, x in zip(rows.tolist(), ci.tolist(), v.tolist()):
            f.write(f"{r + 1} {c + 1} {x!r}\n")
