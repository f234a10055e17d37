"""Matrix ingestion for the drivers: the file formats of the reference's
example programs (README:101-118) read into CSR on the host and built into
a device operator (propack_csr_create, or propack_zcsr_create for complex
data: upload, device transpose, SpMV schedule).

* Harwell-Boeing, assembled (``.rua``, ``.rsa``, ``.rra``, ``.cua``,
  ``.csa``, ``.cha``, ``.pua``, ...; ``.hb``, ``.rb``): real, complex and
  pattern matrices, unsymmetric, rectangular, symmetric, Hermitian and
  skew-symmetric.  The reference's test matrices are illc1850.rra (real)
  and mhd1280b.cua (complex, README:105-107); scipy.io.hb_read reads no
  complex files, so this module parses the format itself: the header's
  card counts, type and Fortran data formats, then fixed-width fields;
* Matrix Market coordinate or array (``.mtx``), real or complex --
  scipy.io.mmread;
* coordinate ASCII (``.coord``): one ``i j a`` triple per line (``i j re
  im`` for complex data), 1-based, optionally preceded by an ``m n nnz``
  line;
* dense ASCII (``.dense``): ``m n`` then the m*n values, column by column
  (Fortran order, as the reference's programs store arrays), or m*n
  (re, im) pairs for complex data;
* diagonal ASCII (``.diag``): ``m n ndiag``, then per stored diagonal its
  offset d (entries A(i, i+d)) followed by its min(m, n-d) - max(0, -d)
  values in order of increasing row.  The reference's example reader for
  this format is not in its source tree (README:113-118 names it), so this
  is the plain DIA layout its name describes.
Symmetric, Hermitian and skew-symmetric input is expanded to the full
matrix.
"""
import os
import re

import numpy as np
import scipy.sparse as sp

from . import CsrOperator


HB_EXTENSIONS = tuple(k + s + "a" for k in "rcp" for s in "usrhz") + ("hb", "rb")


def read(path, fmt=None):
    """The matrix in ``path`` as a scipy CSR array (float64, or complex128
    when the file holds complex values)."""
    fmt = (fmt or os.path.splitext(path)[1].lstrip(".")).lower()
    if fmt in HB_EXTENSIONS:
        A = read_harwell_boeing(path)
    elif fmt == "mtx":
        from scipy.io import mmread
        try:
            A = mmread(path, spmatrix=False)
        except TypeError:  # a scipy that predates the argument
            A = mmread(path)
    elif fmt == "coord":
        A = _read_coord(path)
    elif fmt == "dense":
        A = _read_dense(path)
    elif fmt == "diag":
        A = _read_diag(path)
    else:
        raise ValueError(f"unknown matrix format {fmt!r}")
    A = sp.csr_array(A, dtype=np.complex128 if np.iscomplexobj(_values(A)) else np.float64)
    A.sum_duplicates()
    return A


def _values(A):
    return A.data if sp.issparse(A) else np.asarray(A)


# ------------------------------------------------------------ Harwell-Boeing
def _fortran_format(fmt):
    """(fields per line, field width, integer?) of a data format such as
    (26I3), (1P,4E20.12), (1P4D16.8) or (5F15.8)."""
    f = fmt.strip().upper().replace(" ", "")
    if f.startswith("(") and f.endswith(")"):
        f = f[1:-1]
    f = re.sub(r"^-?\d*P,?", "", f)  # a scale factor (1P) does not change the fields
    m = re.fullmatch(r"(\d*)([IEDFG])(\d+)(?:\.\d+)?(?:E\d+)?", f)
    if not m:
        raise ValueError(f"unsupported Fortran data format {fmt!r}")
    return int(m.group(1) or 1), int(m.group(3)), m.group(2) == "I"


def _fortran_real(field):
    t = field.upper().replace("D", "E")
    if "E" not in t:
        # a three-digit exponent written without its letter: 1.0-100
        t = re.sub(r"(?<=[0-9.])([+-]\d+)$", r"E\1", t)
    return float(t)


def _hb_fields(lines, count, fmt):
    """The first ``count`` fields of the card images ``lines``."""
    per, width, is_int = _fortran_format(fmt)
    out = []
    for line in lines:
        for q in range(per):
            field = line[q * width:(q + 1) * width].strip()
            if field:
                out.append(field)
            if len(out) == count:
                break
        if len(out) == count:
            break
    if len(out) < count:
        raise ValueError("Harwell-Boeing file ends inside a data block")
    if is_int:
        return np.array([int(x) for x in out], dtype=np.int64)
    return np.array([_fortran_real(x) for x in out])


def read_harwell_boeing(path):
    """An assembled Harwell-Boeing matrix (Duff, Grimes and Lewis' exchange
    format: title card, card counts, type + shape, Fortran formats, an
    optional right-hand-side card, then 1-based column pointers, row
    indices and values by columns; complex values as (re, im) pairs).
    Symmetric (S), Hermitian (H) and skew-symmetric (Z) files store one
    triangle and are expanded."""
    with open(path) as f:
        lines = f.read().splitlines()
    counts = [int(x) for x in lines[1].split()]
    ptrcrd, indcrd, valcrd = counts[1], counts[2], counts[3]
    rhscrd = counts[4] if len(counts) > 4 else 0
    mxtype = lines[2][:3].upper()
    nrow, ncol, nnz = (int(x) for x in lines[2][3:].split()[:3])
    if len(mxtype) != 3 or mxtype[0] not in "RCP" or mxtype[1] not in "USHZR" or mxtype[2] not in "AE":
        raise ValueError(f"not a Harwell-Boeing type: {mxtype!r}")
    if mxtype[2] != "A":
        raise ValueError("elemental Harwell-Boeing matrices are not supported")
    ptrfmt, indfmt, valfmt = lines[3][0:16], lines[3][16:32], lines[3][32:52]
    p0 = 5 if rhscrd > 0 else 4
    ptr = _hb_fields(lines[p0:p0 + ptrcrd], ncol + 1, ptrfmt) - 1
    i0 = p0 + ptrcrd
    idx = _hb_fields(lines[i0:i0 + indcrd], nnz, indfmt) - 1
    v0 = i0 + indcrd
    if mxtype[0] == "P":
        val = np.ones(nnz)
    elif mxtype[0] == "C":
        v = _hb_fields(lines[v0:v0 + valcrd], 2 * nnz, valfmt)
        val = v[0::2] + 1j * v[1::2]
    else:
        val = _hb_fields(lines[v0:v0 + valcrd], nnz, valfmt)
    if ptr[0] != 0 or ptr[-1] != nnz or np.any(np.diff(ptr) < 0):
        raise ValueError("Harwell-Boeing column pointers are not monotone from 1 to nnz+1")
    if nnz and (idx.min() < 0 or idx.max() >= nrow):
        raise ValueError("Harwell-Boeing row index out of range")
    A = sp.csc_array((val, idx, ptr), shape=(nrow, ncol))
    if mxtype[1] in "SHZ":
        D = sp.diags_array(A.diagonal(), shape=A.shape)
        T = A.T.conj() if mxtype[1] == "H" else A.T
        A = A + T - D if mxtype[1] != "Z" else A - T
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
    ncol = len(rows[0]) if rows else 3
    t = np.array(rows, dtype=np.float64).reshape(-1, ncol)
    i = t[:, 0].astype(np.int64) - 1
    j = t[:, 1].astype(np.int64) - 1
    if shape is None:
        shape = (int(i.max()) + 1, int(j.max()) + 1)
    vals = t[:, 2] + 1j * t[:, 3] if ncol == 4 else t[:, 2]
    return sp.coo_array((vals, (i, j)), shape=shape)


def _read_dense(path):
    with open(path) as f:
        v = np.array(f.read().split(), dtype=np.float64)
    m, n = int(v[0]), int(v[1])
    if v.size - 2 == 2 * m * n:
        z = v[2:].reshape(-1, 2)
        return (z[:, 0] + 1j * z[:, 1]).reshape((m, n), order="F")
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
