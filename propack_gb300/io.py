"""Matrix ingestion for the drivers: the file formats of the reference's
example programs (README:101-118) read into CSR on the host and built into
a device operator (propack_csr_create: upload, device transpose, SpMV
schedule).

* Harwell-Boeing (``.rra``, ``.rua``, ``.rsa``, ``.hb``; the format of the
  reference's test matrix illc1850.rra) -- scipy.io.hb_read;
* Matrix Market coordinate or array (``.mtx``) -- scipy.io.mmread;
* coordinate ASCII (``.coord``): one ``i j a`` triple per line, 1-based,
  optionally preceded by an ``m n nnz`` line;
* dense ASCII (``.dense``): ``m n`` then the m*n values, column by column
  (Fortran order, as the reference's programs store arrays);
* diagonal ASCII (``.diag``): ``m n ndiag``, then per stored diagonal its
  offset d (entries A(i, i+d)) followed by its min(m, n-d) - max(0, -d)
  values in order of increasing row.  The reference's example reader for
  this format is not in its source tree (README:113-118 names it), so this
  is the plain DIA layout its name describes.
Symmetric Harwell-Boeing / Matrix Market input is expanded to both
triangles by the scipy readers.
"""
import os

import numpy as np
import scipy.sparse as sp

from . import CsrOperator


def read(path, fmt=None):
    """The matrix in ``path`` as a scipy CSR array (FP64)."""
    fmt = (fmt or os.path.splitext(path)[1].lstrip(".")).lower()
    if fmt in ("rra", "rua", "rsa", "hb", "rb"):
        from scipy.io import hb_read
        A = hb_read(path)
    elif fmt == "mtx":
        from scipy.io import mmread
        A = mmread(path)
    elif fmt == "coord":
        A = _read_coord(path)
    elif fmt == "dense":
        A = _read_dense(path)
    elif fmt == "diag":
        A = _read_diag(path)
    else:
        raise ValueError(f"unknown matrix format {fmt!r}")
    A = sp.csr_array(A, dtype=np.float64)
    A.sum_duplicates()
    return A


def _read_coord(path):
    rows = []
    with open(path) as f:
        for line in f:
            t = line.split()
            if t and not t[0].startswith(("%", "#")):
                rows.append(t)
    shape = None
    if rows and len(rows[0]) == 3 and all(x.lstrip("-").isdigit() for x in rows[0]) and len(rows) > 1:
        first = [int(x) for x in rows[0]]
        if first[2] == len(rows) - 1:
            shape = (first[0], first[1])
            rows = rows[1:]
    t = np.array(rows, dtype=np.float64).reshape(-1, 3)
    i = t[:, 0].astype(np.int64) - 1
    j = t[:, 1].astype(np.int64) - 1
    if shape is None:
        shape = (int(i.max()) + 1, int(j.max()) + 1)
    return sp.coo_array((t[:, 2], (i, j)), shape=shape)


def _read_dense(path):
    with open(path) as f:
        v = np.array(f.read().split(), dtype=np.float64)
    m, n = int(v[0]), int(v[1])
    return v[2:2 + m * n].reshape((m, n), order="F")


def _read_diag(path):
    with open(path) as f:
        v = f.read().split()
    m, n, nd = int(v[0]), int(v[1]), int(v[2])
    pos, rows, cols, vals = 3, [], [], []
    for _ in range(nd):
        d = int(float(v[pos]))
        pos += 1
        i0, i1 = max(0, -d), min(m, n - d)
        cnt = max(0, i1 - i0)
        i = np.arange(i0, i0 + cnt)
        rows.append(i)
        cols.append(i + d)
        vals.append(np.array(v[pos:pos + cnt], dtype=np.float64))
        pos += cnt
    cat = lambda a, t: np.concatenate(a).astype(t) if a else np.zeros(0, t)
    return sp.coo_array((cat(vals, np.float64), (cat(rows, np.int64), cat(cols, np.int64))), shape=(m, n))


def load(path, fmt=None):
    """A device operator (``CsrOperator``) for the matrix in ``path``."""
    return CsrOperator(read(path, fmt))


__all__ = ["read", "load"]
