"""Failure paths of the device drivers, injected on the host (no GPU fault,
trap or hang is provoked): a user APROD that returns NaN or Inf, a Lanczos
dimension too small to converge, an operator with no nonzeros, the
no-vectors jobs, and the reference's complex example at scipy's test size.
Each mirrors an oracle test that runs on CPU (tests/test_oracle.py)."""
import numpy as np
import pytest
from scipy.sparse.linalg import LinearOperator

import propack_gb300 as pg
from conftest import csr_from, mhd1280b

pytestmark = pytest.mark.gpu


def _poisoned(mode):
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

    return LinearOperator(A.shape, matvec=mv, rmatvec=rmv, dtype=np.float64), cnt


@pytest.mark.timeout(120)
@pytest.mark.parametrize("mode", ["nan_after_5", "inf", "nan_always"])
@pytest.mark.parametrize("irl", [True, False])
def test_nonfinite_user_aprod_ends_without_converged_triplets(mode, irl):
    """A host APROD that starts returning NaN (after 5 products, or from
    the first) or Inf: both drivers return (every data-dependent loop on the
    device is bounded by a count, dlanbpro.F:372-409 takes the
    invariant-subspace path at most a bounded number of times) and claim no
    converged triplet."""
    lo, cnt = _poisoned(mode)
    m, n = lo.shape
    k, kmax = 5, 20
    u = np.zeros((m, kmax + 1), order="F")
    v = np.zeros((n, kmax), order="F")
    u[:, 0] = np.random.default_rng(0).uniform(size=m)
    sig, bnd = np.zeros(k), np.zeros(k)
    iop = np.array([0, 1], dtype=np.int32)
    aprod = pg._host_aprod(lo)
    if irl:
        dop = np.array([np.sqrt(np.finfo(float).eps), np.finfo(float).eps ** 0.75, 0.0, 0.002])
        kc, info = pg.lansvd_irl(b"L", b"y", b"y", m, n, kmax, kmax - k, k, 50, aprod, u, sig, bnd, v, 1e-8,
                                 dop, iop)
    else:
        dop = np.array([np.sqrt(np.finfo(float).eps), np.finfo(float).eps ** 0.75, 0.0])
        kc, info = pg.lansvd(b"y", b"y", m, n, k, kmax, aprod, u, sig, bnd, v, 1e-8, dop, iop)
    assert info != 0 or kc < k, (info, kc, sig)
    assert kc < k
    assert cnt[0] < 1000


def test_kmax_too_small_gives_info_minus_one(golden):
    """dlansvd with a Lanczos dimension too small for the requested
    accuracy ends with INFO = -1 (double/dlansvd.F:250-259)."""
    A = csr_from(golden, "plain")
    op = pg.CsrOperator(A)
    m, n = A.shape
    k, kmax = 10, 12
    u = np.zeros((m, kmax + 1), order="F")
    v = np.zeros((n, kmax), order="F")
    u[:, 0] = np.random.default_rng(0).uniform(size=m)
    sig, bnd = np.zeros(k), np.zeros(k)
    dop = np.array([np.sqrt(np.finfo(float).eps), np.finfo(float).eps ** 0.75, 0.0])
    kc, info = pg.lansvd(b"y", b"y", m, n, k, kmax, op.aprod, u, sig, bnd, v, 1e-12, dop,
                         np.array([0, 1], dtype=np.int32), iparm=op.iparm)
    op.close()
    assert info == -1
    with pytest.raises(Exception, match="did not converge"):
        pg.svdp(A, k, irl_mode=False, kmax=kmax, tol=1e-12, rng=np.random.default_rng(0))


@pytest.mark.parametrize("irl", [True, False])
def test_zero_operator_gives_k_zero_values(irl):
    """An operator with no nonzeros: every start vector is annihilated and
    both drivers report k zero singular values with INFO = 0, as scipy's
    packaging of the reference does."""
    import scipy.sparse as sp
    Z = sp.csr_array((50, 30))
    u, s, vt, bnd = pg.svdp(Z, 3, irl_mode=irl, kmax=10, rng=np.random.default_rng(0))
    np.testing.assert_array_equal(s, np.zeros(3))


@pytest.mark.parametrize("irl", [True, False])
def test_no_vectors_jobs(golden, irl):
    """jobu = jobv = 'n': the same singular values without the Ritz
    vectors (dritzvec is skipped)."""
    A = csr_from(golden, "plain")
    ref = golden["plain_irl_sigma"] if irl else golden["plain_lansvd_sigma"]
    kw = dict(irl_mode=True, kmax=30, tol=1e-12) if irl else dict(irl_mode=False, tol=1e-12)
    u, s, vt, bnd = pg.svdp(A, len(ref), compute_u=False, compute_v=False, rng=np.random.default_rng(0), **kw)
    np.testing.assert_allclose(s, ref, rtol=1e-10)
    assert not np.any(vt)  # V is never written


def test_complex_reference_example_mhd1280b_k200():
    """zlansvd_ on the device, on the reference's complex example matrix at
    scipy's test configuration (k = 200): singular values to 1e-10 of the
    dense SVD and orthonormal leading vectors, as scipy's test checks."""
    A = mhd1280b()
    if A is None:
        pytest.skip("scipy's PROPACK test data is not installed")
    u, s, vh, bnd = pg.svdp(A, 200, irl_mode=False, rng=np.random.default_rng(0))
    dense = np.linalg.svd(A.toarray(), compute_uv=False)
    np.testing.assert_allclose(s, dense[:200], rtol=1e-10)
    c = 27
    np.testing.assert_allclose(u[:, :c].conj().T @ u[:, :c], np.eye(c), atol=1e-9)
    np.testing.assert_allclose(vh[:c] @ vh[:c].conj().T, np.eye(c), atol=1e-9)
