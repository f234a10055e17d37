"""The oracle (CPU restatement of PROPACK) pinned against the reference's
outputs: scipy's packaging of PROPACK (golden fixtures), dense LAPACK, and
the generator table of LAPACK's dlaruv."""
import os

import numpy as np
import pytest

import oracle
from conftest import csr_from, illc1850, subspace_err


def test_lcg_matches_dlaruv_table():
    # rows 1, 2, 3, 4, 64, 117, 128 of dlaruv's multiplier table (base-4096 digits)
    table = {1: (494, 322, 2508, 2549), 2: (2637, 789, 3754, 1145), 3: (255, 1440, 1766, 2253),
             4: (2008, 752, 3572, 305), 64: (2770, 1238, 1956, 2817), 117: (2785, 1832, 1836, 3365),
             128: (545, 2366, 3801, 1537)}
    a = 33952834046453
    for i, dig in table.items():
        x = pow(a, i, 2 ** 48)
        assert ((x >> 36) & 4095, (x >> 24) & 4095, (x >> 12) & 4095, x & 4095) == dig


@pytest.mark.parametrize("n", [1, 2, 3, 10, 57, 150])
def test_bdsqr_vs_numpy(n):
    rng = np.random.default_rng(n)
    d = rng.standard_normal(n)
    e = rng.standard_normal(n - 1)
    B = np.diag(d) + np.diag(e, 1)
    s_ref = np.linalg.svd(B, compute_uv=False)
    dd, U, VT, info = oracle.bdsqr(d, e, nru_vectors=True, ncvt_vectors=True)
    assert info == 0
    np.testing.assert_allclose(dd, s_ref, rtol=1e-13, atol=1e-14 * s_ref[0])
    np.testing.assert_allclose(U @ np.diag(dd) @ VT, B, atol=1e-13 * s_ref[0])
    np.testing.assert_allclose(U.T @ U, np.eye(n), atol=1e-13)
    # last row of the left vectors, as used for the Ritz bounds
    urow = np.zeros(n)
    urow[-1] = 1.0
    d2, U2, _, _ = oracle.bdsqr(d, e, urow=urow)
    np.testing.assert_allclose(np.abs(U2[0]), np.abs(U[-1]), atol=1e-12)


def test_bdsqr_graded_relative_accuracy():
    d = 10.0 ** (-np.arange(20.0))
    e = 10.0 ** (-np.arange(19.0) - 0.5)
    B = np.diag(d) + np.diag(e, 1)
    s_ref = np.linalg.svd(B, compute_uv=False)
    dd, _, _, _ = oracle.bdsqr(d, e)
    np.testing.assert_allclose(dd, s_ref, rtol=1e-12)


def test_plain_lansvd_vs_golden(golden):
    A = csr_from(golden, "plain")
    u, s, vt, bnd, info, kc = oracle.svdp(A, 10, irl_mode=False, kmax=200, tol=1e-12,
                                          rng=np.random.default_rng(0))
    assert info == 0 and kc == 10
    np.testing.assert_allclose(s, golden["plain_lansvd_sigma"], rtol=1e-12)
    np.testing.assert_allclose(s, golden["plain_dense_sigma"][:10], rtol=1e-12)
    assert subspace_err(u, golden["plain_lansvd_u"]) < 1e-10
    assert subspace_err(vt.T, golden["plain_lansvd_vt"].T) < 1e-10


def test_plain_irl_vs_golden(golden):
    A = csr_from(golden, "plain")
    u, s, vt, bnd, info, kc = oracle.svdp(A, 10, irl_mode=True, kmax=30, tol=1e-12,
                                          rng=np.random.default_rng(0))
    st = oracle.getstat()
    oracle.clearstat()
    assert info == 0 and kc == 10
    assert st["nrestart"] > 0
    np.testing.assert_allclose(s, golden["plain_irl_sigma"], rtol=1e-12)
    assert subspace_err(u, golden["plain_irl_u"]) < 1e-9


@pytest.mark.parametrize("case,kw", [("small_irl_lm", dict(irl_mode=True, which="LM")),
                                     ("small_irl_sm", dict(irl_mode=True, which="SM")),
                                     ("small_lansvd", dict(irl_mode=False))])
def test_small_cases_vs_golden(golden, case, kw):
    A = csr_from(golden, "small")
    which = kw.pop("which", "LM")
    u, s, vt, bnd, info, kc = oracle.svdp(A.toarray(), 3, which=which, tol=1e-8, rng=np.random.default_rng(0), **kw)
    assert info == 0
    np.testing.assert_allclose(s, golden[case + "_sigma"], rtol=1e-8, atol=1e-8)


def test_lowrank_irl_vs_golden(golden):
    S, L, R = csr_from(golden, "lr_S"), csr_from(golden, "lr_L"), csr_from(golden, "lr_R")
    w = golden["lr_w"]
    op = oracle.Operator(S, L, R, w)
    u, s, vt, bnd, info, kc = oracle.svdp(None, 10, irl_mode=True, kmax=30, tol=1e-10,
                                          rng=np.random.default_rng(0), op=op)
    assert info == 0 and kc == 10
    np.testing.assert_allclose(s, golden["lowrank_irl_sigma"], rtol=1e-10)
    np.testing.assert_allclose(s, golden["lowrank_dense_sigma"][:10], rtol=1e-10)


def test_python_callback_equals_builtin_operator(golden):
    A = csr_from(golden, "plain")
    r1 = oracle.svdp(A, 10, irl_mode=False, kmax=200, tol=1e-12, rng=np.random.default_rng(0))
    from scipy.sparse.linalg import aslinearoperator
    r2 = oracle.svdp(aslinearoperator(A), 10, irl_mode=False, kmax=200, tol=1e-12, rng=np.random.default_rng(0))
    np.testing.assert_allclose(r1[1], r2[1], rtol=1e-13)


@pytest.mark.slow
def test_illc1850_vs_golden(golden):
    A = illc1850()
    if A is None or "illc_sigma" not in golden:
        pytest.skip("illc1850 not available")
    u, s, vt, bnd, info, kc = oracle.svdp(A, 200, irl_mode=False, rng=np.random.default_rng(0))
    assert info == 0
    np.testing.assert_allclose(s, golden["illc_sigma"], rtol=1e-11)
    np.testing.assert_allclose(u.T @ u, np.eye(200), atol=1e-9)
    np.testing.assert_allclose(vt @ vt.T, np.eye(200), atol=1e-9)


def test_operator_does_not_modify_its_inputs(golden):
    S, L, R = csr_from(golden, "lr_S"), csr_from(golden, "lr_L"), csr_from(golden, "lr_R")
    before = [a.copy() for a in (S.data, S.indices, S.indptr, L.data, R.data)]
    oracle.Operator(S, L, R, golden["lr_w"])
    after = (S.data, S.indices, S.indptr, L.data, R.data)
    assert all(np.array_equal(x, y) for x, y in zip(before, after))


def test_mlp_oracle_gradient_matches_finite_differences():
    """The CPU oracle of the learned start model: its backward pass (in FP64)
    against central differences of its own loss."""
    import oracle.mlp_oracle as mo
    rng = np.random.default_rng(0)
    F = rng.standard_normal((300, 18))
    U, _ = np.linalg.qr(rng.standard_normal((300, 5)))
    p = mo.init_params(1)
    p[mo.OB1:mo.OW2] = 0.1
    p[mo.OB2:mo.OW3] = 0.1
    _, g = mo.loss_and_grad(p, F, U, bf=False)
    h = 1e-6
    for i in list(rng.integers(0, mo.NP, 24)) + [mo.OB3, mo.OW3, mo.OB1, mo.OB2]:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss_and_grad(pp, F, U, bf=False)[0] - mo.loss_and_grad(pm, F, U, bf=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * (abs(g[i]) + 1e-3)


def test_bf16_rounding_of_the_mlp_oracle():
    import oracle.mlp_oracle as mo
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], dtype=np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] - (-3.140625)) < 1e-7 and r[4] == 0.0


def test_matrix_file_formats_round_trip(tmp_path):
    """propack_gb300.io reads the example programs' formats back exactly."""
    import scipy.io as sio
    import scipy.sparse as sp
    from propack_gb300 import io as pio
    rng = np.random.default_rng(3)
    A = sp.random_array((40, 25), density=0.2, format="csr", random_state=rng)
    A = sp.csr_array(A)
    p = tmp_path / "a.mtx"
    sio.mmwrite(str(p), A)
    assert np.array_equal(pio.read(str(p)).toarray(), A.toarray())
    p = tmp_path / "a.rua"
    sio.hb_write(str(p), sp.csc_array(A))
    np.testing.assert_allclose(pio.read(str(p)).toarray(), A.toarray(), rtol=1e-15, atol=0)
    C = A.tocoo()
    p = tmp_path / "a.coord"
    with open(p, "w") as f:
        f.write(f"{A.shape[0]} {A.shape[1]} {C.nnz}\n")
        for i, j, v in zip(C.row, C.col, C.data):
            f.write(f"{i + 1} {j + 1} {float(v)!r}\n")
    assert np.array_equal(pio.read(str(p)).toarray(), A.toarray())
    D = A.toarray()
    p = tmp_path / "a.dense"
    with open(p, "w") as f:
        f.write(f"{D.shape[0]} {D.shape[1]}\n")
        f.write("\n".join(repr(float(x)) for x in D.ravel(order="F")))
    assert np.array_equal(pio.read(str(p)).toarray(), D)
    # banded matrix in the diagonal format (offsets -2, 0, 3; a wide shape)
    m, n = 12, 17
    B = np.zeros((m, n))
    p = tmp_path / "a.diag"
    with open(p, "w") as f:
        f.write(f"{m} {n} 3\n")
        for d in (-2, 0, 3):
            i = np.arange(max(0, -d), min(m, n - d))
            vals = rng.standard_normal(i.size)
            B[i, i + d] = vals
            f.write(f"{d} " + " ".join(repr(float(x)) for x in vals) + "\n")
    assert np.array_equal(pio.read(str(p)).toarray(), B)


# ------------------------------------------------------------------ complex
GOLDEN_Z = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_complex.npz")


def _zgolden():
    with np.load(GOLDEN_Z, allow_pickle=False) as d:
        return {k: d[k] for k in d.files}


def _zcsr(g, prefix):
    import scipy.sparse as sp
    shape = tuple(int(x) for x in g[prefix + "_shape"])
    return sp.csr_array((g[prefix + "_data"].copy(), g[prefix + "_indices"].copy(), g[prefix + "_indptr"].copy()),
                        shape=shape)


@pytest.mark.parametrize("case,mat,k,kw", [("z1_lansvd", "z1", 5, dict(kmax=80)),
                                           ("z1_lansvd_cgs", "z1", 5, dict(kmax=80, cgs=True)),
                                           ("z2_lansvd", "z2", 6, dict(kmax=120))])
def test_complex_oracle_matches_scipy_zlansvd(case, mat, k, kw):
    """The complex*16 restatement (zlanbpro, zreorth, zlansvd) against
    scipy's packaging of PROPACK's zlansvd on the same inputs: singular
    values, bounds and vectors."""
    import oracle
    g = _zgolden()
    A = _zcsr(g, mat)
    u, s, vh, bnd, info, kc = oracle.svdp(A, k, irl_mode=False, tol=1e-12, rng=np.random.default_rng(0), **kw)
    assert info == 0 and kc == k
    np.testing.assert_allclose(s, g[case + "_sigma"], rtol=1e-12)
    np.testing.assert_allclose(s, g[mat + "_dense_sigma"][:k], rtol=1e-12)
    # the bounds follow the same Lanczos trajectory (tiny ones are rounding noise)
    np.testing.assert_allclose(bnd, g[case + "_bnd"], rtol=1e-6, atol=1e-14 * s[0])
    assert np.max(np.abs(np.abs(np.sum(u.conj() * g[case + "_u"], axis=0)) - 1)) < 1e-10
    assert np.max(np.abs(np.abs(np.sum(vh.conj() * g[case + "_vh"], axis=1)) - 1)) < 1e-10


@pytest.mark.parametrize("kmax,cgs", [(12, False), (30, False), (30, True)])
def test_complex_oracle_irl_matches_dense(kmax, cgs):
    """zlansvd_irl restated: restarts with the real shifts and rotations of B
    applied to the complex bases.  Pinned to the dense SVD (scipy's
    complex IRL returns wrong values on this input, see make_golden_complex)."""
    import oracle
    g = _zgolden()
    A = _zcsr(g, "z1")
    oracle.clearstat()
    u, s, vh, bnd, info, kc = oracle.svdp(A, 5, irl_mode=True, kmax=kmax, tol=1e-12, cgs=cgs,
                                          rng=np.random.default_rng(0))
    stt = oracle.getstat()
    assert info == 0 and kc == 5
    if kmax == 12:
        assert stt["nrestart"] > 0
    np.testing.assert_allclose(s, g["z1_dense_sigma"][:5], rtol=1e-12)
    Ad = A.toarray()
    res = max(np.linalg.norm(Ad @ vh[i].conj() - s[i] * u[:, i]) for i in range(5))
    assert res < 1e-10 * s[0]
    # scipy's restarted complex driver is off on this input (recorded)
    assert np.max(np.abs(g["z1_irl_scipy_sigma"] - g["z1_dense_sigma"][:5])) > 0.1


def test_complex_oracle_random_start():
    """A zero start vector: zgetu0 draws the real and imaginary parts from
    dlaruv's stream (zlarnv, idist 2)."""
    import oracle
    g = _zgolden()
    A = _zcsr(g, "z2")
    u, s, vh, bnd, info, kc = oracle.svdp(A, 4, irl_mode=True, kmax=24, tol=1e-12,
                                          v0=np.zeros(A.shape[0], dtype=np.complex128))
    assert info == 0 and kc == 4
    np.testing.assert_allclose(s, g["z2_dense_sigma"][:4], rtol=1e-12)


def test_complex_oracle_on_the_reference_example_mhd1280b():
    """zlansvd restated on PROPACK's complex example matrix (1280 x 1280),
    against scipy's packaging of the reference at scipy's own test
    configuration (k=200; orthogonality and reconstruction of the leading
    27 triplets as scipy checks them) and, for the restarted driver at
    k=50, kmax=120 (converged without a restart), against scipy's values,
    which miss the same copies of the repeated singular value 2."""
    from conftest import mhd1280b
    import oracle
    A = mhd1280b()
    if A is None:
        pytest.skip("scipy's PROPACK test data is not installed")
    g = _zgolden()
    u, s, vh, bnd, info, kc = oracle.svdp(A, 200, irl_mode=False, rng=np.random.default_rng(0))
    assert info == 0 and kc == 200
    np.testing.assert_allclose(s, g["mhd_lansvd_sigma"], rtol=1e-12)
    np.testing.assert_allclose(s, g["mhd_dense_sigma"], rtol=1e-12)
    c = 27
    np.testing.assert_allclose(u[:, :c].conj().T @ u[:, :c], np.eye(c), atol=1e-9)
    np.testing.assert_allclose(vh[:c] @ vh[:c].conj().T, np.eye(c), atol=1e-9)
    u3, s3, vh3 = np.linalg.svd(A.toarray())
    recon = (u[:, :c] * s[:c]) @ vh[:c] - (u3[:, :c] * s3[:c]) @ vh3[:c]
    assert np.linalg.norm(recon) < 1e-9
    oracle.clearstat()
    u, s, vh, bnd, info, kc = oracle.svdp(A, 50, irl_mode=True, kmax=120, tol=1e-10, rng=np.random.default_rng(0))
    assert info == 0 and kc == 50 and oracle.getstat()["nrestart"] == 0
    np.testing.assert_allclose(s, g["mhd_irl50_sigma"], rtol=1e-12)
    assert np.sum(np.abs(s - g["mhd_dense_sigma"][:50]) > 1e-8) > 0


@pytest.mark.timeout(60)
@pytest.mark.parametrize("mode", ["nan_after_5", "inf", "nan_always"])
@pytest.mark.parametrize("irl", [True, False])
def test_nonfinite_aprod_terminates(mode, irl):
    """Failure injection on the host: an APROD that returns NaN or Inf ends
    the restated drivers (the control flow the device drivers share: every
    data-dependent loop is bounded) with no converged triplet claimed."""
    from scipy.sparse.linalg import LinearOperator
    import oracle
    A = np.random.default_rng(0).random((60, 40))
    cnt = [0]

    def poison(y, i):
        if mode == "inf":
            y[i] = np.inf
        elif mode == "nan_always" or cnt[0] > 5:
            y[i] = np.nan
        return y

    def mv(x):
        cnt[0] += 1
        return poison(A @ x, 0)

    def rmv(x):
        cnt[0] += 1
        return poison(A.T @ x, 1)

    lo = LinearOperator(A.shape, matvec=mv, rmatvec=rmv, dtype=np.float64)
    u, s, vt, bnd, info, kc = oracle.svdp(lo, 5, irl_mode=irl, kmax=20, maxiter=50, rng=np.random.default_rng(0))
    assert kc < 5 and cnt[0] < 200


@pytest.mark.parametrize("irl", [True, False])
def test_zero_matrix_matches_scipy(irl):
    """An operator with no nonzeros: every start vector is annihilated, the
    bidiagonal is zero, and both drivers report k zero singular values with
    INFO = 0, as scipy's packaging of the reference does."""
    import scipy.sparse as sp
    from scipy.sparse.linalg._svdp import _svdp
    import oracle
    Z = sp.csr_array((50, 30))
    u, s, vt, bnd, info, kc = oracle.svdp(Z, 3, irl_mode=irl, kmax=10, rng=np.random.default_rng(0))
    ref = _svdp(Z, 3, irl_mode=irl, kmax=10, rng=np.random.default_rng(0))[1]
    assert info == 0 and kc == 3
    np.testing.assert_array_equal(s, ref)
    np.testing.assert_array_equal(s, np.zeros(3))
