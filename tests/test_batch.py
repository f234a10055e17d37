"""The batched persistent-kernel solver against the oracle, problem by
problem (same start vectors; full reorthogonalisation with classical
Gram-Schmidt on both sides)."""
import numpy as np
import pytest

import oracle
from conftest import subspace_err
from propack_gb300 import batch

pytestmark = pytest.mark.gpu


def _oracle(A, k, kmax, tol, u0):
    uo, so, vto, bo, info, kc = oracle.svdp(A, k, kmax=kmax, tol=tol, v0=u0, cgs=True, delta=0.0, eta=0.0,
                                            rng=np.random.default_rng(0))
    return uo, so, vto.T, info


@pytest.mark.parametrize("kmax,k", [(16, 4), (24, 8)])
def test_batch_matches_dense_svd(kmax, k):
    """Converged to tol = 1e-12, every problem's triplets agree with LAPACK's
    dense SVD: values to 1e-10 relative, vectors to a sin-angle of 1e-8."""
    mats = batch.random_batch(20, m_range=(300, 1500), n_range=(100, 600), density=0.03, seed=5)
    rng = np.random.default_rng(1)
    u0 = [rng.uniform(size=A.shape[0]) for A in mats]
    B = batch.Batch(mats)
    sig, bnd, info, U, V = B.solve(k, kmax=kmax, tol=1e-12, maxiter=200, u0=u0)
    st = B.stats
    assert st["cycles"] >= 1 and st["grid"] >= 1 and st["converged"] + st["fallback"] == len(mats)
    for p, A in enumerate(mats):
        assert info[p] == 0
        Ud, sd, Vdt = np.linalg.svd(A.toarray(), full_matrices=False)
        np.testing.assert_allclose(sig[p], sd[:k], rtol=1e-10)
        assert subspace_err(U[p], Ud[:, :k]) < 1e-8
        assert subspace_err(V[p], Vdt[:k].T) < 1e-8
    B.close()


def test_batch_vs_oracle_at_tol_1e8():
    """At tol = 1e-8 the batched kernel follows the oracle's Lanczos
    trajectory: the same values and vectors, residuals within tol."""
    mats = batch.random_batch(12, m_range=(300, 1500), n_range=(100, 600), density=0.03, seed=8)
    rng = np.random.default_rng(4)
    u0 = [rng.uniform(size=A.shape[0]) for A in mats]
    B = batch.Batch(mats)
    k, kmax = 6, 20
    sig, bnd, info, U, V = B.solve(k, kmax=kmax, tol=1e-8, maxiter=60, u0=u0)
    for p, A in enumerate(mats):
        assert info[p] == 0
        uo, so, vo, io = _oracle(A, k, kmax, 1e-8, u0[p])
        assert io == 0
        # the same Lanczos trajectory as the oracle's, up to rounding
        np.testing.assert_allclose(sig[p], so, rtol=1e-10)
        assert subspace_err(U[p], uo) < 1e-8
        assert subspace_err(V[p], vo) < 1e-8
        res = max(np.linalg.norm(A @ V[p][:, i] - sig[p, i] * U[p][:, i]) for i in range(k))
        assert res < 1e-8 * sig[p, 0]
        assert np.all(bnd[p] <= 1e-8 * sig[p])
    B.close()


def test_batch_uneven_sizes_single_call():
    """One call over problems whose sizes differ by two orders of magnitude."""
    rng = np.random.default_rng(2)
    mats = batch.random_batch(6, m_range=(200, 300), n_range=(80, 120), density=0.05, seed=6)
    mats += batch.random_batch(2, m_range=(6000, 8000), n_range=(2000, 3000), density=0.005, seed=7)
    u0 = [rng.uniform(size=A.shape[0]) for A in mats]
    B = batch.Batch(mats)
    sig, bnd, info, U, V = B.solve(6, kmax=20, tol=1e-8, maxiter=80, u0=u0)
    for p, A in enumerate(mats):
        assert info[p] == 0
        s_ref = np.linalg.svd(A.toarray(), compute_uv=False)[:6]
        np.testing.assert_allclose(sig[p], s_ref, rtol=1e-10)
    B.close()


def test_autotuner_table_and_pinned_choices():
    """The autotuner times its candidates once per batch; every choice of the
    table solves correctly; the projection tile dc changes no bit, and a
    pinned table gives the same bits on every solve."""
    mats = batch.random_batch(24, m_range=(300, 3000), n_range=(100, 900), density=0.02, seed=9)
    rng = np.random.default_rng(3)
    u0 = [rng.uniform(size=A.shape[0]) for A in mats]
    dense = [np.linalg.svd(A.toarray(), compute_uv=False)[:6] for A in mats]
    B = batch.Batch(mats)
    assert B.tuning()["state"] == 0
    sig, bnd, info, U, V = B.solve(6, kmax=20, tol=1e-12, maxiter=200, u0=u0, vectors=False)
    t = B.tuning()
    assert t["state"] == 1 and B.stats["tune_ms"] > 0
    assert all(g in (1, 4, 8, 32) for g in t["g"]) and all(d in (1, 2, 4) for d in t["dc"])
    assert all(b <= d * 1.0001 for b, d in zip(t["probe_ms"], t["probe_ms_default"]))
    for p in range(len(mats)):
        np.testing.assert_allclose(sig[p], dense[p], rtol=1e-10)
    sig2, _, _, _, _ = B.solve(6, kmax=20, tol=1e-12, maxiter=200, u0=u0, vectors=False)
    assert B.stats["tune_ms"] == 0.0 and np.array_equal(sig, sig2)
    out = {}
    for g, dc in ((1, 1), (1, 4), (32, 2), (8, 1)):
        B.set_tuning([g] * batch.NCLASS, [dc] * batch.NCLASS)
        assert B.tuning()["state"] == 2
        out[(g, dc)] = B.solve(6, kmax=20, tol=1e-12, maxiter=200, u0=u0, vectors=False)[0]
        for p in range(len(mats)):
            np.testing.assert_allclose(out[(g, dc)][p], dense[p], rtol=1e-10)
    assert np.array_equal(out[(1, 1)], out[(1, 4)])
    B.set_tuning()
    assert B.tuning()["state"] == 0
    B.close()


def test_plane_and_fp64_arithmetics_agree():
    """The batched kernel's FP32-plane products and Gram-Schmidt passes
    (propack_batch_set_arith(h, 2)) against its FP64 ones (the default) on
    the same batch: every problem converges, values agree to 1e-10 and with
    LAPACK's, and the matvec counts stay close (the two differ by rounding
    only)."""
    mats = batch.random_batch(16, m_range=(300, 3000), n_range=(100, 900), density=0.02, seed=12)
    rng = np.random.default_rng(6)
    u0 = [rng.uniform(size=A.shape[0]) for A in mats]
    out = {}
    for arith in ("planes", "fp64"):
        B = batch.Batch(mats)
        B.set_arith(arith)
        B.set_tuning([1] * batch.NCLASS, [1] * batch.NCLASS)
        sig, bnd, info, U, V = B.solve(6, kmax=20, tol=1e-10, maxiter=200, u0=u0, vectors=True)
        out[arith] = (sig, info, U, V, B.stats["nopx"])
        B.close()
    (s1, i1, U1, V1, n1), (s2, i2, U2, V2, n2) = out["planes"], out["fp64"]
    assert np.all(i1 == 0) and np.all(i2 == 0)
    for p, A in enumerate(mats):
        np.testing.assert_allclose(s1[p], s2[p], rtol=1e-10)
        np.testing.assert_allclose(s1[p], np.linalg.svd(A.toarray(), compute_uv=False)[:6], rtol=1e-9)
        assert subspace_err(U1[p], U2[p]) < 1e-7 and subspace_err(V1[p], V2[p]) < 1e-7
    assert abs(n1 - n2) <= 0.1 * n2
