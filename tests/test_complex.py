"""The complex*16 drivers (zlansvd_, zlansvd_irl_ through the C ABI) against
the complex oracle and scipy's zlansvd outputs (tests/golden/golden_complex.npz).

The device holds a complex operator natively (complex CSR and its
conjugate transpose, complex SpMV) or, on request, as its real 2x2-block
form; the CPU tests pin the block form (propack_zcsr_expand, host code)
against complex products, and a GPU test holds the two forms to each other.  GPU tolerances are those of the FP64 path: singular values 1e-10
relative, phase-free vector agreement | |<u_gpu, u_ref>| - 1 | < 1e-8,
operator products 1e-12 relative."""
import ctypes as C
import os

import numpy as np
import pytest
import scipy.sparse as sp
from scipy.sparse.linalg import LinearOperator

import oracle
import propack_gb300 as pg

GOLDEN_Z = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_complex.npz")
SIG_RTOL = 1e-10
VEC_TOL = 1e-8


def zgolden():
    with np.load(GOLDEN_Z, allow_pickle=False) as d:
        return {k: d[k] for k in d.files}


def zcsr(g, prefix):
    shape = tuple(int(x) for x in g[prefix + "_shape"])
    return sp.csr_array((g[prefix + "_data"].copy(), g[prefix + "_indices"].copy(), g[prefix + "_indptr"].copy()),
                        shape=shape)


def ragged_complex(seed, m, n):
    """Complex CSR with empty rows, single entries and a few long rows."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 6, m)
    lens[rng.random(m) < 0.25] = 0
    lens[rng.choice(m, 3, replace=False)] = rng.integers(n // 2, n, 3)
    ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    idx = np.concatenate([np.sort(rng.choice(n, k, replace=False)) for k in lens]).astype(np.int32)
    val = rng.standard_normal(ptr[-1]) + 1j * rng.standard_normal(ptr[-1])
    return sp.csr_array((val, idx, ptr), shape=(m, n))


def geometric_complex(seed=1, m=240, n=160, r=60, q=0.5):
    """A = X diag(q^i) Y^H with random orthonormal complex X, Y: a fast-
    decaying spectrum on which the extended local reorthogonalisation runs
    (zlanbpro.F:318-331, :451-464)."""
    rng = np.random.default_rng(seed)
    X, _ = np.linalg.qr(rng.standard_normal((m, r)) + 1j * rng.standard_normal((m, r)))
    Y, _ = np.linalg.qr(rng.standard_normal((n, r)) + 1j * rng.standard_normal((n, r)))
    return sp.csr_array((X * q ** np.arange(r)) @ Y.conj().T)


def phase_err(a, b, axis=0):
    """max | |<a_i, b_i>| - 1 | over matched columns (axis 0) or rows (axis 1)."""
    return float(np.max(np.abs(np.abs(np.sum(a.conj() * b, axis=axis)) - 1.0)))


def expand(A):
    L = pg.load()
    m, n = A.shape
    ptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
    idx = np.ascontiguousarray(A.indices, dtype=np.int32)
    val = np.ascontiguousarray(A.data, dtype=np.complex128)
    nnz = int(ptr[-1])
    p2 = np.zeros(2 * m + 1, dtype=np.int64)
    i2 = np.zeros(max(4 * nnz, 1), dtype=np.int32)
    v2 = np.zeros(max(4 * nnz, 1))
    rc = L.propack_zcsr_expand(m, n, pg._i64p(ptr), pg._ip(idx), C.c_void_p(val.ctypes.data), pg._i64p(p2),
                               pg._ip(i2), pg._dp(v2))
    return rc, sp.csr_array((v2[:4 * nnz], i2[:4 * nnz], p2), shape=(2 * m, 2 * n))


def pairs(z):
    return np.ascontiguousarray(z, dtype=np.complex128).view(np.float64)


# ------------------------------------------------------------------ CPU
def test_zcsr_expand_is_the_2x2_block_form():
    """Each entry b + ic becomes [b -c; c b] on the (re, im) pairs: the real
    form applied to pairs gives A x, its transpose gives A^H y."""
    A = ragged_complex(7, 57, 41)
    rc, R = expand(A)
    assert rc == 0
    rng = np.random.default_rng(1)
    x = rng.standard_normal(41) + 1j * rng.standard_normal(41)
    y = rng.standard_normal(57) + 1j * rng.standard_normal(57)
    np.testing.assert_allclose(R @ pairs(x), pairs(A @ x), rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(R.T @ pairs(y), pairs(A.conj().T @ y), rtol=1e-13, atol=1e-13)
    D, B = A.toarray(), R.toarray()
    np.testing.assert_array_equal(B[0::2, 0::2], D.real)
    np.testing.assert_array_equal(B[0::2, 1::2], -D.imag)
    np.testing.assert_array_equal(B[1::2, 0::2], D.imag)
    np.testing.assert_array_equal(B[1::2, 1::2], D.real)
    # row order is kept: the entries of each real row follow row i of A
    assert all(np.all(np.diff(R.indices[R.indptr[r]:R.indptr[r + 1]]) > 0) for r in range(2 * 57))


def test_zcsr_expand_rejects_bad_input():
    A = ragged_complex(3, 20, 10)
    bad_ptr = A.copy()
    bad_ptr.indptr = A.indptr.copy()
    bad_ptr.indptr[5], bad_ptr.indptr[6] = bad_ptr.indptr[6] + 1, bad_ptr.indptr[5]
    assert expand(bad_ptr)[0] == pg.ERR_ARG
    bad_col = A.copy()
    bad_col.indices = A.indices.copy()
    bad_col.indices[bad_col.nnz // 2] = 10
    assert expand(bad_col)[0] == pg.ERR_ARG
    neg_col = A.copy()
    neg_col.indices = A.indices.copy()
    neg_col.indices[0] = -1
    assert expand(neg_col)[0] == pg.ERR_ARG


def test_complex_test_matrices_run_the_elr_in_the_oracle():
    """The GPU cases below reach the complex ELR kernels: the oracle takes
    ELR passes on the same inputs."""
    g = zgolden()
    for A, kw in [(geometric_complex(), dict(k=6, kmax=40, irl_mode=False)),
                  (zcsr(g, "z1"), dict(k=5, kmax=12, irl_mode=True)),
                  (zcsr(g, "z2"), dict(k=6, kmax=120, irl_mode=False))]:
        oracle.clearstat()
        oracle.svdp(A, tol=1e-12, rng=np.random.default_rng(0), **kw)
        assert oracle.nelr() > 0


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("which", ["ragged", "z1"])
def test_complex_operator_products(which):
    A = ragged_complex(11, 3001, 700) if which == "ragged" else zcsr(zgolden(), "z1")
    op = pg.CsrOperator(A)
    assert op.dtype == np.complex128
    m, n = A.shape
    rng = np.random.default_rng(2)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = rng.standard_normal(m) + 1j * rng.standard_normal(m)
    ref_n, ref_c = A @ x, A.conj().T @ y
    got_n, got_c = op.matvec(x), op.rmatvec(y)
    np.testing.assert_allclose(got_n, ref_n, rtol=1e-12, atol=1e-12 * np.abs(ref_n).max())
    np.testing.assert_allclose(got_c, ref_c, rtol=1e-12, atol=1e-12 * np.abs(ref_c).max())
    op.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case,mat,k,kw", [("z1_lansvd", "z1", 5, dict(kmax=80)),
                                           ("z1_lansvd_cgs", "z1", 5, dict(kmax=80, cgs=True)),
                                           ("z2_lansvd", "z2", 6, dict(kmax=120))])
def test_complex_lansvd_matches_oracle_and_scipy(case, mat, k, kw):
    """zlansvd_ on the device operator: the oracle's trajectory and scipy's
    zlansvd outputs (values, bounds, vectors up to phase)."""
    g = zgolden()
    A = zcsr(g, mat)
    u, s, vh, bnd = pg.svdp(A, k, irl_mode=False, tol=1e-12, rng=np.random.default_rng(0), **kw)
    st = pg.get_stats()
    uo, so, vho, bo, info, kc = oracle.svdp(A, k, irl_mode=False, tol=1e-12, rng=np.random.default_rng(0), **kw)
    assert info == 0 and kc == k
    np.testing.assert_allclose(s, so, rtol=SIG_RTOL)
    np.testing.assert_allclose(s, g[case + "_sigma"], rtol=SIG_RTOL)
    # converged by PROPACK's test; the bounds themselves are rounding-level
    assert np.all(bnd <= 1e-12 * s)
    np.testing.assert_allclose(bnd, g[case + "_bnd"], rtol=0, atol=1e-12 * s[0])
    assert phase_err(u, uo) < VEC_TOL and phase_err(u, g[case + "_u"]) < VEC_TOL
    assert phase_err(vh, vho, axis=1) < VEC_TOL and phase_err(vh, g[case + "_vh"], axis=1) < VEC_TOL
    oracle.clearstat()
    oracle.svdp(A, k, irl_mode=False, tol=1e-12, rng=np.random.default_rng(0), **kw)
    no = oracle.getstat()["nopx"]
    assert abs(st["nopx"] - no) <= 0.05 * no + 4


@pytest.mark.gpu
@pytest.mark.parametrize("kmax,cgs", [(12, False), (30, False), (30, True)])
def test_complex_irl_matches_oracle_and_dense(kmax, cgs):
    """zlansvd_irl_: restarts with real shifts and rotations applied to the
    complex bases on the tensor-core GEMM's real (re, im) rows."""
    g = zgolden()
    A = zcsr(g, "z1")
    u, s, vh, bnd = pg.svdp(A, 5, irl_mode=True, kmax=kmax, tol=1e-12, cgs=cgs, rng=np.random.default_rng(0))
    st = pg.get_stats()
    uo, so, vho, bo, info, kc = oracle.svdp(A, 5, irl_mode=True, kmax=kmax, tol=1e-12, cgs=cgs,
                                            rng=np.random.default_rng(0))
    np.testing.assert_allclose(s, g["z1_dense_sigma"][:5], rtol=SIG_RTOL)
    np.testing.assert_allclose(s, so, rtol=SIG_RTOL)
    assert phase_err(u, uo) < VEC_TOL and phase_err(vh, vho, axis=1) < VEC_TOL
    Ad = A.toarray()
    res = max(np.linalg.norm(Ad @ vh[i].conj() - s[i] * u[:, i]) for i in range(5))
    assert res < 1e-10 * s[0]
    if kmax == 12:
        assert st["nrestart"] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("irl", [False, True])
def test_complex_elr_matches_oracle(irl):
    """A fast-decaying spectrum, where the complex ELR (its projection
    kernel and its update passes) runs in most steps."""
    A = geometric_complex()
    kw = dict(kmax=40, tol=1e-12, irl_mode=irl)
    u, s, vh, bnd = pg.svdp(A, 6, rng=np.random.default_rng(0), **kw)
    uo, so, vho, bo, info, kc = oracle.svdp(A, 6, rng=np.random.default_rng(0), **kw)
    np.testing.assert_allclose(s, so, rtol=SIG_RTOL)
    np.testing.assert_allclose(s, np.linalg.svd(A.toarray(), compute_uv=False)[:6], rtol=SIG_RTOL)
    assert phase_err(u, uo) < VEC_TOL and phase_err(vh, vho, axis=1) < VEC_TOL


@pytest.mark.gpu
def test_complex_tensor_core_restarts():
    """4100 complex rows are 8200 real rows: the restart and Ritz products
    run on the tcgen05 GEMM (4096 rows and up), applied to (re, im) rows."""
    A = ragged_complex(5, 4100, 600)
    kw = dict(irl_mode=True, kmax=24, tol=1e-10)
    u, s, vh, bnd = pg.svdp(A, 5, rng=np.random.default_rng(0), **kw)
    st = pg.get_stats()
    uo, so, vho, bo, info, kc = oracle.svdp(A, 5, rng=np.random.default_rng(0), **kw)
    assert info == 0 and kc == 5 and st["nrestart"] > 0
    np.testing.assert_allclose(s, so, rtol=SIG_RTOL)
    assert phase_err(u, uo) < VEC_TOL and phase_err(vh, vho, axis=1) < VEC_TOL
    res = max(np.linalg.norm(A @ vh[i].conj() - s[i] * u[:, i]) for i in range(5))
    assert res < 1e-9 * s[0]


@pytest.mark.gpu
def test_complex_host_zaprod_matches_device_operator():
    """A complex LinearOperator goes through the host ZAPROD ('n', 'c') and
    follows the same trajectory as the device operator."""
    g = zgolden()
    A = zcsr(g, "z2")
    lo = LinearOperator(A.shape, matvec=lambda x: A @ x, rmatvec=lambda y: A.conj().T @ y, dtype=np.complex128)
    kw = dict(irl_mode=True, kmax=30, tol=1e-12)
    u1, s1, vh1, b1 = pg.svdp(A, 4, rng=np.random.default_rng(0), **kw)
    n1 = pg.get_stats()["nopx"]
    u2, s2, vh2, b2 = pg.svdp(lo, 4, rng=np.random.default_rng(0), **kw)
    n2 = pg.get_stats()["nopx"]
    np.testing.assert_allclose(s2, s1, rtol=SIG_RTOL)
    np.testing.assert_allclose(s1, g["z2_dense_sigma"][:4], rtol=SIG_RTOL)
    assert phase_err(u1, u2) < VEC_TOL
    assert abs(n1 - n2) <= 2 * 30


@pytest.mark.gpu
def test_complex_zero_start_and_smallest():
    """A zero start vector (zgetu0: real and imaginary parts from dlaruv's
    stream) and which='SM'."""
    g = zgolden()
    A = zcsr(g, "z2")
    z0 = np.zeros(A.shape[0], dtype=np.complex128)
    u, s, vh, bnd = pg.svdp(A, 4, irl_mode=True, kmax=24, tol=1e-12, v0=z0, rng=np.random.default_rng(0))
    uo, so, vho, bo, info, kc = oracle.svdp(A, 4, irl_mode=True, kmax=24, tol=1e-12, v0=z0)
    np.testing.assert_allclose(s, so, rtol=SIG_RTOL)
    np.testing.assert_allclose(s, g["z2_dense_sigma"][:4], rtol=SIG_RTOL)
    assert phase_err(u, uo) < VEC_TOL
    # which='SM' with p <= dim/2 (larger p is the reference's known
    # restart problem for the smallest values, Changelog:56) and full
    # reorthogonalisation (delta = 0): with the partial scheme the oracle
    # itself returns spurious tiny values on 2 of 40 random draws of this
    # family (seeds 8 and 25), and the draw depends on the host's LAPACK
    B = geometric_complex(seed=2, m=120, n=90, r=90, q=0.97)
    kw = dict(which='SM', irl_mode=True, kmax=60, shifts=20, tol=1e-10, maxiter=800, delta=0.0)
    u, s, vh, bnd = pg.svdp(B, 3, rng=np.random.default_rng(0), **kw)
    uo, so, vho, bo, info, kc = oracle.svdp(B, 3, rng=np.random.default_rng(0), **kw)
    dense = np.linalg.svd(B.toarray(), compute_uv=False)
    np.testing.assert_allclose(np.sort(s), np.sort(dense[-3:]), rtol=1e-8)
    np.testing.assert_allclose(s, so, rtol=1e-8)


@pytest.mark.gpu
def test_complex_operator_is_refused_by_the_real_drivers():
    A = zcsr(zgolden(), "z1")
    op = pg.CsrOperator(A)
    m, n = A.shape
    u = np.zeros((m, 11), order='F')
    u[:, 0] = 1.0
    v = np.zeros((n, 10), order='F')
    sig, bnd = np.zeros(3), np.zeros(3)
    dop = np.array([1e-8, 1e-12, 0.0, 0.002])
    iop = np.array([0, 1], dtype=np.int32)
    aprod = C.cast(pg.load().propack_gpu_csr_aprod_, pg.APROD)
    kc, info = pg.lansvd_irl(b'L', b'y', b'y', m, n, 10, 5, 3, 10, aprod, u, sig, bnd, v, 1e-8, dop, iop,
                             iparm=op.iparm)
    assert info == pg.ERR_ARG
    assert "complex" in pg.last_error()
    op.close()


@pytest.mark.gpu
def test_native_and_block_forms_agree():
    """The native complex operator (complex CSR, complex SpMV that also
    forms the ELR's complex projection) against the real 2x2-block form on
    the same matrices: products to 1e-12, the same zlansvd_irl_ results and
    matvec counts within rounding, and one ELR launch fewer per triggered
    ELR step in the native form (same ELR passes)."""
    rng = np.random.default_rng(3)
    out = {}
    for form in ("native", "block"):
        pg.set_complex_form(form)
        try:
            ops = [pg.CsrOperator(ragged_complex(11, 3001, 700)), pg.CsrOperator(geometric_complex())]
        finally:
            pg.set_complex_form("native")
        res = []
        for op in ops:
            m, n = op.shape
            x = np.random.default_rng(5).standard_normal(n) + 1j * np.random.default_rng(6).standard_normal(n)
            y = np.random.default_rng(7).standard_normal(m) + 1j * np.random.default_rng(8).standard_normal(m)
            prods = (op.matvec(x), op.rmatvec(y))
            pg.set_profiling(True)
            u, s, vh, bnd = pg.svdp(op, 6, irl_mode=True, kmax=40, tol=1e-12, rng=np.random.default_rng(0))
            prof = pg.get_profile()
            pg.set_profiling(False)
            res.append((prods, s, u, vh, pg.get_stats(), prof))
            op.close()
        out[form] = res
    for (pn, sn, un, vn, stn, prn), (pb, sb, ub, vb, stb, prb), A in zip(
            out["native"], out["block"], (ragged_complex(11, 3001, 700), geometric_complex())):
        for got, ref in zip(pn, pb):
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
        np.testing.assert_allclose(sn, sb, rtol=SIG_RTOL)
        np.testing.assert_allclose(sn, np.linalg.svd(A.toarray(), compute_uv=False)[:6], rtol=SIG_RTOL)
        assert phase_err(un, ub) < VEC_TOL and phase_err(vn, vb, axis=1) < VEC_TOL
        assert abs(stn["nopx"] - stb["nopx"]) <= 0.05 * stb["nopx"] + 4
    # the block form enqueues one more ELR launch per half step (the pass
    # that forms the complex projection)
    prn, prb = out["native"][1][5], out["block"][1][5]
    assert 0 < prn["elr"][0] < prb["elr"][0]


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["native", "block"])
def test_complex_plane_gram_schmidt_agrees_with_fp64(form):
    """The complex Gram-Schmidt passes on FP32 (hi, lo) planes (the default)
    against the complex FP64 kernels (propack_set_cgs_arith(0)), with both
    operator forms: values to 1e-12, the same vectors up to phase, matvec
    counts within a restart; the plane kernels stream columns."""
    g = zgolden()
    cases = [(zcsr(g, "z1"), 5, dict(irl_mode=True, kmax=30, tol=1e-12, cgs=True)),
             (geometric_complex(), 6, dict(irl_mode=True, kmax=40, tol=1e-12)),
             (ragged_complex(5, 4100, 600), 5, dict(irl_mode=True, kmax=24, tol=1e-10))]
    pg.set_complex_form(form)
    try:
        ops = [(pg.CsrOperator(A), k, kw) for A, k, kw in cases]
    finally:
        pg.set_complex_form("native")
    try:
        for op, k, kw in ops:
            out = {}
            for arith in ("fp64", "planes"):
                pg.set_cgs_arith(arith)
                u, s, vh, bnd = pg.svdp(op, k, rng=np.random.default_rng(0), **kw)
                out[arith] = (u, s, vh, pg.get_stats())
            (u0, s0, vh0, st0), (u1, s1, vh1, st1) = out["fp64"], out["planes"]
            np.testing.assert_allclose(s1, s0, rtol=1e-12)
            assert phase_err(u1, u0) < VEC_TOL and phase_err(vh1, vh0, axis=1) < VEC_TOL
            assert abs(st1["nopx"] - st0["nopx"]) <= 2 * kw["kmax"]
            assert st1["cgs_cols_u"] + st1["cgs_cols_v"] > 0
            op.close()
    finally:
        pg.set_cgs_arith("planes")


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["native", "block"])
def test_complex_zero_and_tiny_operators(form):
    """Edge cases of both operator forms: an operator with no nonzeros
    annihilates every start vector and both drivers report k zero values
    (INFO 0, as the real drivers and scipy's packaging do); a 7 x 5 dense
    complex matrix (rows shorter and longer than a warp's run) gives the
    oracle's values.  There the reference itself stops 4e-8 (sigma_1) and
    2.6e-6 (sigma_2) from LAPACK's values -- scipy's packaging of PROPACK
    returns the same -- so the comparison is with the oracle."""
    rng = np.random.default_rng(9)
    Z = sp.csr_array((50, 30), dtype=np.complex128)
    D = sp.csr_array(rng.standard_normal((7, 5)) + 1j * rng.standard_normal((7, 5)))
    pg.set_complex_form(form)
    try:
        for irl in (True, False):
            u, s, vh, bnd = pg.svdp(Z, 3, irl_mode=irl, kmax=10, rng=np.random.default_rng(0))
            np.testing.assert_array_equal(s, np.zeros(3))
            u, s, vh, bnd = pg.svdp(D, 2, irl_mode=irl, kmax=5, tol=1e-12, rng=np.random.default_rng(0))
            so = oracle.svdp(D, 2, irl_mode=irl, kmax=5, tol=1e-12, rng=np.random.default_rng(0))[1]
            np.testing.assert_allclose(s, so, rtol=1e-10)
            np.testing.assert_allclose(s, np.linalg.svd(D.toarray(), compute_uv=False)[:2], rtol=1e-5)
    finally:
        pg.set_complex_form("native")
