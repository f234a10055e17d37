"""Matrix files (propack_gb300.io): the Harwell-Boeing reader against scipy's
reader on real files and against hand-written complex / symmetric /
Hermitian / skew / pattern files, and complex data through the Matrix
Market, coordinate and dense readers (host code), and, on the GPU, the
device operator built from files of each kind."""
import numpy as np
import pytest
import scipy.io as sio
import scipy.sparse as sp

from propack_gb300 import io as pio

# A = [[1+2i, 0, 3-i], [0, 4, 0], [5+0.5i, 0, 6-6i]], complex unsymmetric
# assembled, by columns; values with a 1P scale factor and D exponents
CUA_3x3 = """\
Complex 3x3 test matrix                                                 CUA3
             5             1             1             3             0
CUA                        3             3             5             0
(4I3)           (5I3)           (1P,4D16.8)
  1  3  4  6
  1  3  2  1  3
  1.00000000D+00  2.00000000D+00  5.00000000D+00  5.00000000D-01
  4.00000000D+00  0.00000000D+00  3.00000000D+00 -1.00000000D+00
  6.00000000D+00 -6.00000000D+00
"""
CUA_DENSE = np.array([[1 + 2j, 0, 3 - 1j], [0, 4, 0], [5 + 0.5j, 0, 6 - 6j]])

# Hermitian, lower triangle stored: [[2, 1-i], [1+i, 3]]
CHA_2x2 = """\
Hermitian                                                               CHA2
             4             1             1             2             0
CHA                        2             2             3             0
(3I4)           (3I4)           (4E15.7)
   1   3   4
   1   2   2
  2.0000000E+00  0.0000000E+00  1.0000000E+00  1.0000000E+00
  3.0000000E+00  0.0000000E+00
"""

# real symmetric [[4, 1], [1, 5]] with a right-hand-side card present (its
# data after the values is not part of the matrix)
RSA_2x2_RHS = """\
Symmetric with rhs                                                      RSA2
             5             1             1             1             1
RSA                        2             2             3             0
(3I4)           (3I4)           (3F10.4)            (3F10.4)
F                          1             0
   1   3   4
   1   2   2
    4.0000    1.0000    5.0000
    9.0000    9.0000
"""

# real skew-symmetric [[0, -2.5], [2.5, 0]]: the strict lower triangle;
# the value has a three-digit exponent written without its letter
RZA_2x2 = """\
Skew                                                                    RZA2
             3             1             1             1             0
RZA                        2             2             1             0
(3I4)           (3I4)           (1E16.8)
   1   2   2
   2
  2.50000000+000
"""

# pattern, unsymmetric rectangular 2x3: entries (1,1), (2,2), (1,3)
PRA_2x3 = """\
Pattern                                                                 PRA
             2             1             1             0             0
PRA                        2             3             3             0
(4I3)           (3I3)
  1  2  3  4
  1  2  1
"""


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_harwell_boeing_real_files_match_scipys_reader(tmp_path):
    for seed in range(4):
        rng = np.random.default_rng(seed)
        A = sp.random_array((37 + seed, 23), density=0.3, format="csc", random_state=rng)
        p = str(tmp_path / f"a{seed}.rua")
        sio.hb_write(p, A)
        assert np.array_equal(pio.read(p).toarray(), sp.csr_array(sio.hb_read(p)).toarray())


@pytest.mark.parametrize("name,text,dense", [
    ("a.cua", CUA_3x3, CUA_DENSE),
    ("a.cha", CHA_2x2, np.array([[2, 1 - 1j], [1 + 1j, 3]])),
    ("a.rsa", RSA_2x2_RHS, np.array([[4.0, 1.0], [1.0, 5.0]])),
    ("a.rza", RZA_2x2, np.array([[0.0, -2.5], [2.5, 0.0]])),
    ("a.pra", PRA_2x3, np.array([[1.0, 0.0, 1.0], [0.0, 1.0, 0.0]])),
])
def test_harwell_boeing_types(tmp_path, name, text, dense):
    A = pio.read(write(tmp_path, name, text))
    assert A.dtype == (np.complex128 if np.iscomplexobj(dense) else np.float64)
    np.testing.assert_array_equal(A.toarray(), dense)


def test_harwell_boeing_rejects_broken_files(tmp_path):
    short = CUA_3x3.rsplit("\n", 2)[0] + "\n"  # the last value card is missing
    with pytest.raises(ValueError):
        pio.read(write(tmp_path, "s.cua", short))
    bad_row = CUA_3x3.replace("  1  3  2  1  3", "  1  3  2  1  4")
    with pytest.raises(ValueError):
        pio.read(write(tmp_path, "r.cua", bad_row))
    elemental = CUA_3x3.replace("CUA                        3", "CUE                        3")
    with pytest.raises(ValueError):
        pio.read(write(tmp_path, "e.cue", elemental), fmt="hb")


def test_complex_matrix_market_coordinate_and_dense(tmp_path):
    rng = np.random.default_rng(5)
    A = sp.random_array((19, 13), density=0.3, format="coo", random_state=rng)
    A = sp.coo_array((A.data + 1j * rng.standard_normal(A.nnz), (A.row, A.col)), shape=A.shape)
    p = str(tmp_path / "z.mtx")
    sio.mmwrite(p, A)
    R = pio.read(p)
    assert R.dtype == np.complex128
    np.testing.assert_array_equal(R.toarray(), A.toarray())
    p = tmp_path / "z.coord"
    with open(p, "w") as f:
        f.write(f"{A.shape[0]} {A.shape[1]} {A.nnz}\n")
        for i, j, v in zip(A.row, A.col, A.data):
            f.write(f"{i + 1} {j + 1} {float(v.real)!r} {float(v.imag)!r}\n")
    np.testing.assert_array_equal(pio.read(str(p)).toarray(), A.toarray())
    D = A.toarray()
    p = tmp_path / "z.dense"
    with open(p, "w") as f:
        f.write(f"{D.shape[0]} {D.shape[1]}\n")
        f.write("\n".join(f"{float(z.real)!r} {float(z.imag)!r}" for z in D.ravel(order="F")))
    np.testing.assert_array_equal(pio.read(str(p)).toarray(), D)


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", ["mtx", "rua", "coord", "complex_mtx"])
def test_device_operator_from_a_matrix_file(tmp_path, fmt):
    """io.load builds the device operator from a file (upload, device
    checks and transposition, SpMV schedule): its products equal scipy's on
    the matrix read back, and a solve on it gives the dense SVD's values."""
    import propack_gb300 as pg
    rng = np.random.default_rng(11)
    m, n = 300, 180
    A = sp.csr_array(sp.random_array((m, n), density=0.05, format="csr", random_state=rng))
    if fmt == "complex_mtx":
        A = sp.csr_array(A + 1j * sp.csr_array(sp.random_array((m, n), density=0.05, format="csr",
                                                              random_state=rng)))
    # the Matrix Market writer appends ".mtx" to a name without it
    p = tmp_path / ("a.mtx" if fmt.endswith("mtx") else f"a.{fmt}")
    if fmt == "mtx":
        sio.mmwrite(str(p), A)
    elif fmt == "rua":
        sio.hb_write(str(p), sp.csc_array(A))
    elif fmt == "coord":
        C = A.tocoo()
        with open(p, "w") as f:
            f.write(f"{m} {n} {C.nnz}\n")
            for i, j, v in zip(C.row, C.col, C.data):
                f.write(f"{i + 1} {j + 1} {float(v)!r}\n")
    else:
        sio.mmwrite(str(p), A)  # complex data through the Matrix Market reader
    ref = pio.read(str(p))
    op = pio.load(str(p))
    x = rng.standard_normal(n) + (1j * rng.standard_normal(n) if fmt == "complex_mtx" else 0)
    y = rng.standard_normal(m) + (1j * rng.standard_normal(m) if fmt == "complex_mtx" else 0)
    np.testing.assert_allclose(op.matvec(x), ref @ x, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(op.rmatvec(y), ref.conj().T @ y, rtol=1e-12, atol=1e-12)
    u, s, vt, bnd = pg.svdp(op, 5, kmax=40, tol=1e-12, rng=np.random.default_rng(0))
    np.testing.assert_allclose(s, np.linalg.svd(ref.toarray(), compute_uv=False)[:5], rtol=1e-10)
    op.close()
