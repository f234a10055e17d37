"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: every matrix is generated from numpy
``default_rng(seed)`` with the sizes, sparsity patterns and value
distributions of the five solver configurations.

* ``plain_lansvd``   2000 x 1000 CSR, 5 distinct uniform columns per row,
                     N(0,1) values, row i scaled by (1+i)^-0.5 (k=10,
                     kmax=200, tol=1e-12).
* ``lowrank_irl``    m x n CSR with ``nnz_row`` uniform columns per row and
                     N(0,1) values, plus a rank-``rank`` term
                     sum_i w_i u_i v_i' with sparse unit-norm Gaussian u_i
                     (density ``udens``) and v_i (density ``vdens``),
                     w_i = 100 * 0.9^i, kept factored (A = S + L diag(w) R').
                     The full-size case is 2,000,000 x 500,000, 20 nnz/row,
                     rank 64, 1% / 5% densities (k=50, dim=150, tol=1e-10).
                     Duplicate column draws in a row are kept as separate
                     entries; the operator sums them, exactly as a merged
                     entry would.
* ``zipf_mixed``     m x m CSR, nnz per row Zipf(2) clipped to [4, 2000],
                     uniform columns, N(0,1) * (1 + i mod 1000)^-0.7 values.
* ``zipf_complex``   the same pattern with complex values, real and
                     imaginary parts N(0,1) * (1 + i mod 1000)^-0.7 (the
                     complex*16 drivers' workload; no configuration of the
                     reference names a complex one).
"""
import numpy as np
import scipy.sparse as sp


def plain_lansvd(seed=0, m=2000, n=1000, nnz_row=5):
    rng = np.random.default_rng(seed)
    rows = np.repeat(np.arange(m), nnz_row)
    cols = np.concatenate([rng.choice(n, nnz_row, replace=False) for _ in range(m)])
    vals = rng.standard_normal(m * nnz_row)
    vals *= np.repeat((1.0 + np.arange(m)) ** -0.5, nnz_row)
    A = sp.csr_array((vals, (rows, cols)), shape=(m, n))
    A.sort_indices()
    return A


def _uniform_csr(rng, m, n, nnz_row, scale_rows=None):
    nnz = m * nnz_row
    indptr = np.arange(0, nnz + 1, nnz_row, dtype=np.int64)
    indices = rng.integers(0, n, size=nnz, dtype=np.int32)
    data = rng.standard_normal(nnz)
    if scale_rows is not None:
        data *= np.repeat(scale_rows, nnz_row)
    return sp.csr_array((data, indices, indptr), shape=(m, n))


def _sparse_unit_columns(rng, rows, r, dens):
    """rows x r CSR with about dens*rows Gaussian entries per column, each column of unit norm."""
    per = max(1, int(round(dens * rows)))
    cols, ridx, vals = [], [], []
    for i in range(r):
        ri = rng.choice(rows, per, replace=False)
        v = rng.standard_normal(per)
        v /= np.linalg.norm(v)
        ridx.append(ri)
        cols.append(np.full(per, i, dtype=np.int32))
        vals.append(v)
    M = sp.coo_array((np.concatenate(vals), (np.concatenate(ridx), np.concatenate(cols))), shape=(rows, r))
    return sp.csr_array(M)


def lowrank_irl(seed=1, m=2_000_000, n=500_000, nnz_row=20, rank=64, udens=0.01, vdens=0.05):
    """Returns (S, L, R, w) with A = S + L diag(w) R'."""
    rng = np.random.default_rng(seed)
    S = _uniform_csr(rng, m, n, nnz_row)
    L = _sparse_unit_columns(rng, m, rank, udens)
    R = _sparse_unit_columns(rng, n, rank, vdens)
    w = 100.0 * 0.9 ** np.arange(rank)
    return S, L, R, w


def zipf_mixed(seed=2, m=4_000_000, alpha=2.0, lo=4, hi=2000):
    rng = np.random.default_rng(seed)
    counts = np.clip(rng.zipf(alpha, size=m), lo, hi).astype(np.int64)
    indptr = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(counts, out=indptr[1:])
    nnz = int(indptr[-1])
    indices = rng.integers(0, m, size=nnz, dtype=np.int32)
    data = rng.standard_normal(nnz).astype(np.float32)
    rw = (1.0 + (np.arange(m) % 1000)) ** -0.7
    data *= np.repeat(rw, counts).astype(np.float32)
    return sp.csr_array((data.astype(np.float64), indices, indptr), shape=(m, m))


def lowrank_family(seed=4, m=200_000, n=50_000, rank=32, theta=0.05, sigma0=50.0, decay=0.85, nnz_row=10,
                   noise=0.1):
    """A_t = L_t + E_t, t = 0, 1, ...: L_t = X_t diag(sigma0 decay^i) Y_t'
    with orthonormal X_t (m x rank), Y_t (n x rank) that a random Givens
    sweep of angle +-theta over adjacent column pairs rotates at every step;
    E_t sparse noise with nnz_row uniform columns per row, N(0, noise^2).
    Yields (S, L, R, w) for CsrOperator(S, L, R, w) with L = X_t, R = Y_t
    as dense-as-CSR factors and w the singular weights."""
    rng = np.random.default_rng(seed)
    X, _ = np.linalg.qr(rng.standard_normal((m, rank)))
    Y, _ = np.linalg.qr(rng.standard_normal((n, rank)))
    w = sigma0 * decay ** np.arange(rank)

    def sweep(M):
        for j in range(rank - 1):
            a = theta * (1.0 if rng.random() < 0.5 else -1.0)
            c, s = np.cos(a), np.sin(a)
            x, y = M[:, j].copy(), M[:, j + 1].copy()
            M[:, j] = c * x - s * y
            M[:, j + 1] = s * x + c * y
        return M

    t = 0
    while True:
        er = np.random.default_rng((seed, t))
        indptr = np.arange(m + 1, dtype=np.int64) * nnz_row
        E = sp.csr_array((er.standard_normal(m * nnz_row) * noise, er.integers(0, n, size=m * nnz_row,
                                                                                dtype=np.int32), indptr),
                         shape=(m, n))
        yield E, sp.csr_array(X), sp.csr_array(Y), w.copy()
        X = sweep(X)
        Y = sweep(Y)
        t += 1


def dense_of(S, L=None, R=None, w=None):
    A = S.toarray()
    if L is not None:
        A = A + (L.toarray() * w) @ R.toarray().T
    return A


def zipf_complex(seed=5, m=2_000_000, alpha=2.0, lo=4, hi=2000):
    rng = np.random.default_rng(seed)
    counts = np.clip(rng.zipf(alpha, size=m), lo, hi).astype(np.int64)
    indptr = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(counts, out=indptr[1:])
    nnz = int(indptr[-1])
    indices = rng.integers(0, m, size=nnz, dtype=np.int32)
    rw = np.repeat((1.0 + (np.arange(m) % 1000)) ** -0.7, counts)
    data = (rng.standard_normal(nnz) + 1j * rng.standard_normal(nnz)) * rw
    return sp.csr_array((data, indices, indptr), shape=(m, m))
