"""Parity of the GPU library (called through its C ABI) with the oracle and
with the reference's outputs (scipy's PROPACK golden fixtures).

Tolerances (FP64 path): singular values 1e-10 relative, singular vectors
|<u_gpu, u_ref>| within 1e-8 of 1 (sin-angle ~1e-8), operator products
1e-12 relative."""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.sparse.linalg import aslinearoperator

import oracle
import propack_gb300 as pg
from propack_gb300 import workloads
from conftest import csr_from, illc1850, subspace_err

pytestmark = pytest.mark.gpu

SIG_RTOL = 1e-10
VEC_TOL = 1e-8


def rng0():
    return np.random.default_rng(0)


def test_loaded_kernels_are_sm103():
    # the runtime loaded the library's own sm_103a code (no JIT from PTX,
    # no other architecture)
    assert pg.load().propack_kernel_binary_version() == 103


# ------------------------------------------------------------ operator
@pytest.mark.parametrize("kind", ["plain", "lowrank", "zipf", "longcols", "ragged"])
def test_operator_products(kind):
    rng = np.random.default_rng(3)
    if kind == "plain":
        S = workloads.plain_lansvd(0)
        L = R = w = None
        Ad = S.toarray()
    elif kind == "lowrank":
        S, L, R, w = workloads.lowrank_irl(seed=5, m=3000, n=800, nnz_row=7, rank=6, udens=0.05, vdens=0.2)
        Ad = workloads.dense_of(S, L, R, w)
    elif kind == "zipf":
        S = workloads.zipf_mixed(seed=4, m=20000, hi=5000)
        L = R = w = None
        Ad = None
    elif kind == "ragged":
        # short-row schedule edge cases: empty rows, single entries, rows
        # spread over many lanes' runs, a row count that is not a multiple of 32
        m, n = 5003, 4000
        lens = rng.integers(0, 8, m)
        lens[rng.random(m) < 0.2] = 0
        lens[rng.choice(m, 12, replace=False)] = rng.integers(100, 3500, 12)
        ptr = np.concatenate([[0], np.cumsum(lens)])
        idx = np.concatenate([np.sort(rng.choice(n, k, replace=False)) for k in lens]).astype(np.int32)
        S = sp.csr_array((rng.standard_normal(ptr[-1]), idx, ptr), shape=(m, n))
        L = R = w = None
        Ad = S.toarray()
    else:
        # dense columns and long rows: exercises the long-segment transpose and single-row blocks
        m, n = 3000, 50
        X = rng.standard_normal((m, n))
        X[rng.random((m, n)) > 0.9] = 0.0
        S = sp.csr_array(X)
        L = R = w = None
        Ad = S.toarray()
    op = pg.CsrOperator(S, L, R, w)
    m, n = op.shape
    x = rng.standard_normal(n)
    y = rng.standard_normal(m)
    if Ad is not None:
        ref_n, ref_t = Ad @ x, Ad.T @ y
    else:
        ref_n, ref_t = S @ x, S.T @ y
    got_n, got_t = op.matvec(x), op.rmatvec(y)
    np.testing.assert_allclose(got_n, ref_n, rtol=1e-12, atol=1e-12 * np.abs(ref_n).max())
    np.testing.assert_allclose(got_t, ref_t, rtol=1e-12, atol=1e-12 * np.abs(ref_t).max())
    # bit-reproducible: same inputs give the same bits
    assert np.array_equal(op.rmatvec(y), got_t)
    op.close()


@pytest.mark.parametrize("mode", ["chunked", "staged", "tuned", "rule"])
def test_spmv_schedules(mode):
    # every schedule gives the product; the timed choice picks one of them,
    # the default rule the chunked one for these short rows
    rng = np.random.default_rng(11)
    # 1032 tiles of 32 rows: the warp search of the chunked schedule meets
    # a final window of exactly 32 tiles
    S = workloads.zipf_mixed(seed=6, m=33000, hi=3000)
    pg.set_spmv_schedule(mode)
    try:
        op = pg.CsrOperator(S)
    finally:
        pg.set_spmv_schedule("rule")
    sched, timed = op.schedule
    if mode == "rule":
        assert sched == {"fwd": "chunked", "adj": "chunked"} and not timed
    elif mode != "tuned":
        assert sched == {"fwd": mode, "adj": mode} and not timed
    else:
        assert set(timed) == {("fwd", "chunked"), ("fwd", "staged"), ("adj", "chunked"), ("adj", "staged")}
    x, y = rng.standard_normal(S.shape[1]), rng.standard_normal(S.shape[0])
    for got, ref in ((op.matvec(x), S @ x), (op.rmatvec(y), S.T @ y)):
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    op.close()


@pytest.mark.parametrize("case", ["plain_irl", "lowrank"])
def test_cgs_arithmetics_agree(golden, case):
    # the Gram-Schmidt passes on the FP32 pipe (exact three-way splits, or
    # the split-once (hi, lo) planes) give the FP64 result: same matvecs
    # within a restart, sigma to 1e-12, the same subspaces
    if case == "plain_irl":
        A, k, kw = csr_from(golden, "plain"), 10, dict(irl_mode=True, kmax=30, tol=1e-12)
    else:
        S, L, R, w = workloads.lowrank_irl(seed=5, m=6000, n=1500, nnz_row=7, rank=12, udens=0.05, vdens=0.2)
        A, k, kw = pg.CsrOperator(S, L, R, w), 8, dict(irl_mode=True, kmax=40, tol=1e-10)
    out = {}
    try:
        for arith in ("fp64", "f3", "planes"):
            pg.set_cgs_arith(arith)
            u, s, vt, bnd = pg.svdp(A, k, rng=rng0(), **kw)
            out[arith] = (u, s, vt, pg.get_stats())
    finally:
        pg.set_cgs_arith("planes")
    u0, s0, vt0, st0 = out["fp64"]
    for arith in ("f3", "planes"):
        u1, s1, vt1, st1 = out[arith]
        np.testing.assert_allclose(s1, s0, rtol=1e-12)
        assert subspace_err(u1, u0) < 1e-9 and subspace_err(vt1.T, vt0.T) < 1e-9
        assert abs(st1["nopx"] - st0["nopx"]) <= 2 * 30
        assert st1["cgs_cols_u"] + st1["cgs_cols_v"] > 0


# -------------------------------------------------- golden (reference) cases
def test_plain_lansvd_vs_golden(golden):
    A = csr_from(golden, "plain")
    u, s, vt, bnd = pg.svdp(A, 10, irl_mode=False, kmax=200, tol=1e-12, rng=rng0())
    np.testing.assert_allclose(s, golden["plain_lansvd_sigma"], rtol=SIG_RTOL)
    np.testing.assert_allclose(s, golden["plain_dense_sigma"][:10], rtol=SIG_RTOL)
    assert subspace_err(u, golden["plain_lansvd_u"]) < VEC_TOL
    assert subspace_err(vt.T, golden["plain_lansvd_vt"].T) < VEC_TOL


def test_plain_irl_vs_golden(golden):
    A = csr_from(golden, "plain")
    u, s, vt, bnd = pg.svdp(A, 10, irl_mode=True, kmax=30, tol=1e-12, rng=rng0())
    st = pg.get_stats()
    assert st["nrestart"] > 0
    np.testing.assert_allclose(s, golden["plain_irl_sigma"], rtol=SIG_RTOL)
    assert subspace_err(u, golden["plain_irl_u"]) < VEC_TOL
    assert subspace_err(vt.T, golden["plain_irl_vt"].T) < VEC_TOL


@pytest.mark.parametrize("case,kw", [("small_irl_lm", dict(irl_mode=True, which="LM")),
                                     ("small_irl_sm", dict(irl_mode=True, which="SM")),
                                     ("small_lansvd", dict(irl_mode=False))])
@pytest.mark.parametrize("ctor", ["dense", "csr", "linop"])
def test_small_cases_vs_golden(golden, case, kw, ctor):
    M = csr_from(golden, "small").toarray()
    A = {"dense": M, "csr": sp.csr_array(M), "linop": aslinearoperator(M)}[ctor]
    u, s, vt, bnd = pg.svdp(A, 3, tol=1e-8, rng=rng0(), **kw)
    np.testing.assert_allclose(s, golden[case + "_sigma"], rtol=1e-8, atol=1e-8)
    u1, s1, vt1 = np.linalg.svd(M, full_matrices=False)
    if kw.get("which") == "SM":
        u1, vt1 = np.roll(u1, 3, 1), np.roll(vt1, 3, 0)
    np.testing.assert_allclose(np.abs(u1.T @ u), np.eye(10, 3), atol=1e-8)
    np.testing.assert_allclose(np.abs(vt1 @ vt.T), np.eye(10, 3), atol=1e-8)


def test_lowrank_irl_vs_golden(golden):
    S, L, R = csr_from(golden, "lr_S"), csr_from(golden, "lr_L"), csr_from(golden, "lr_R")
    op = pg.CsrOperator(S, L, R, golden["lr_w"])
    u, s, vt, bnd = pg.svdp(op, 10, irl_mode=True, kmax=30, tol=1e-10, rng=rng0())
    np.testing.assert_allclose(s, golden["lowrank_irl_sigma"], rtol=SIG_RTOL)
    np.testing.assert_allclose(s, golden["lowrank_dense_sigma"][:10], rtol=SIG_RTOL)
    # residuals against the operator itself
    res = max(np.linalg.norm(op.matvec(vt[i]) - s[i] * u[:, i]) for i in range(10))
    assert res < 1e-8 * s[0]
    op.close()


def test_illc1850_vs_golden(golden):
    A = illc1850()
    if A is None or "illc_sigma" not in golden:
        pytest.skip("illc1850 not available")
    u, s, vt, bnd = pg.svdp(A, 200, irl_mode=False, rng=rng0())
    np.testing.assert_allclose(s, golden["illc_sigma"], rtol=1e-10)
    np.testing.assert_allclose(u.T @ u, np.eye(200), atol=1e-9)
    np.testing.assert_allclose(vt @ vt.T, np.eye(200), atol=1e-9)


# ----------------------------------------------------- GPU vs oracle, same inputs
OPTS = [dict(), dict(cgs=True), dict(elr=False), dict(delta=1e-20, eta=1e-10),  # full reorthogonalisation
        dict(delta=-1.0, eta=-1.0)]                                           # PROPACK's own defaults


@pytest.mark.parametrize("opts", OPTS, ids=["default", "cgs", "noelr", "full", "propack_defaults"])
@pytest.mark.parametrize("irl", [True, False])
def test_vs_oracle_same_trajectory(golden, opts, irl):
    S, L, R = csr_from(golden, "lr_S"), csr_from(golden, "lr_L"), csr_from(golden, "lr_R")
    w = golden["lr_w"]
    op = pg.CsrOperator(S, L, R, w)
    oop = oracle.Operator(S, L, R, w)
    kw = dict(irl_mode=irl, kmax=30 if irl else 120, tol=1e-10, **opts)
    u, s, vt, bnd = pg.svdp(op, 10, rng=rng0(), **kw)
    st = pg.get_stats()
    oracle.clearstat()
    uo, so, vto, bo, info, kc = oracle.svdp(None, 10, rng=rng0(), op=oop, **kw)
    sto = oracle.getstat()
    assert info == 0 and kc == 10
    np.testing.assert_allclose(s, so, rtol=SIG_RTOL)
    assert subspace_err(u, uo) < VEC_TOL
    assert subspace_err(vt.T, vto.T) < VEC_TOL
    # the same Lanczos trajectory up to rounding: partial reorthogonalisation
    # and the convergence test are threshold decisions, so one restart more or
    # less (2 * shifts matvecs) is within parity
    shifts = kw["kmax"] - 10 if irl else 0
    assert abs(st["nopx"] - sto["nopx"]) <= 0.05 * sto["nopx"] + 2 * shifts + 4
    op.close()


@pytest.mark.parametrize("irl", [True, False])
def test_tall_bases_vs_oracle(irl):
    """m, n >= 4096: the restart and Ritz products run on the tensor cores
    (the FP64 digit-split GEMM); results stay within the FP64 tolerances."""
    S, L, R, w = workloads.lowrank_irl(seed=11, m=9000, n=5000, nnz_row=6, rank=8, udens=0.02, vdens=0.05)
    op = pg.CsrOperator(S, L, R, w)
    oop = oracle.Operator(S, L, R, w)
    kw = dict(irl_mode=irl, kmax=40 if irl else 90, tol=1e-10)
    u, s, vt, bnd = pg.svdp(op, 12, rng=rng0(), **kw)
    uo, so, vto, bo, info, kc = oracle.svdp(None, 12, rng=rng0(), op=oop, **kw)
    assert info == 0 and kc == 12
    np.testing.assert_allclose(s, so, rtol=SIG_RTOL)
    assert subspace_err(u, uo) < VEC_TOL
    assert subspace_err(vt.T, vto.T) < VEC_TOL
    res = max(np.linalg.norm(op.matvec(vt[i]) - s[i] * u[:, i]) for i in range(12))
    assert res < 1e-9 * s[0]
    op.close()


def test_fp32_valued_matrix_vs_oracle():
    """A matrix whose values are all FP32 numbers (the zipf workload's kind):
    the solve matches the oracle on the same trajectory."""
    S = workloads.zipf_mixed(seed=4, m=20000, hi=3000)
    assert np.array_equal(S.data.astype(np.float32).astype(np.float64), S.data)
    op = pg.CsrOperator(S)
    oop = oracle.Operator(S, None, None, None)
    kw = dict(irl_mode=True, kmax=40, tol=1e-10)
    u, s, vt, bnd = pg.svdp(op, 10, rng=rng0(), **kw)
    st = pg.get_stats()
    oracle.clearstat()
    uo, so, vto, bo, info, kc = oracle.svdp(None, 10, rng=rng0(), op=oop, **kw)
    sto = oracle.getstat()
    assert info == 0 and kc == 10
    np.testing.assert_allclose(s, so, rtol=SIG_RTOL)
    assert subspace_err(u, uo) < VEC_TOL and subspace_err(vt.T, vto.T) < VEC_TOL
    assert abs(st["nopx"] - sto["nopx"]) <= 0.05 * sto["nopx"] + 2 * 30 + 4
    op.close()


def test_zero_start_vector_uses_dlarnv(golden):
    """v0 = 0 makes the driver draw PROPACK's own dlarnv start vector (dgetu0)."""
    A = csr_from(golden, "plain")
    z = np.zeros(A.shape[0])
    u, s, vt, bnd = pg.svdp(A, 10, irl_mode=False, kmax=200, tol=1e-12, v0=z, rng=rng0())
    uo, so, vto, bo, info, kc = oracle.svdp(A, 10, irl_mode=False, kmax=200, tol=1e-12, v0=z, rng=rng0())
    np.testing.assert_allclose(s, so, rtol=SIG_RTOL)
    np.testing.assert_allclose(s, golden["plain_dense_sigma"][:10], rtol=SIG_RTOL)


def test_invariant_subspace_rank_deficient():
    """A rank-6 matrix: the Lanczos run meets an invariant subspace
    (dlanbpro.F:372-409 / :503-539) and the drivers report it as the
    reference does."""
    rng = np.random.default_rng(7)
    X = rng.standard_normal((60, 6)) @ rng.standard_normal((6, 40))
    A = sp.csr_array(X)
    res = {}
    for name, fn in (("gpu", lambda: pg.svdp(A, 4, irl_mode=False, kmax=30, tol=1e-10, rng=rng0())),
                     ("oracle", lambda: oracle.svdp(A, 4, irl_mode=False, kmax=30, tol=1e-10, rng=rng0()))):
        try:
            out = fn()
            res[name] = ("ok", out[1])
        except Exception as e:  # LinAlgError on INFO > 0
            res[name] = ("err", type(e).__name__)
    if res["oracle"][0] == "ok":
        assert res["gpu"][0] == "ok"
        np.testing.assert_allclose(res["gpu"][1], np.linalg.svd(X, compute_uv=False)[:4], rtol=1e-10)
    else:
        assert res["gpu"] == res["oracle"]


def test_invalid_csr_is_rejected_on_the_device():
    # the row pointers and column indices are checked on the device before
    # any kernel indexes by them
    import ctypes as C
    L = pg.load()
    m, n = 40, 30
    nul64, nul32, nuld = C.POINTER(C.c_int64)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()

    def create(ptr, idx):
        val = np.ones(idx.size)
        h = C.c_int64(0)
        rc = L.propack_csr_create(m, n, pg._i64p(ptr), pg._ip(idx), pg._dp(val), 0, nul64, nul32, nuld, nul64,
                                  nul32, nuld, nuld, C.byref(h))
        if rc == 0:
            L.propack_csr_destroy(h.value)
        return rc, pg.last_error()

    ptr = np.arange(0, 2 * m + 1, 2, dtype=np.int64)
    idx = np.tile(np.array([0, 5], dtype=np.int32), m)
    assert create(ptr, idx)[0] == 0
    bad = idx.copy()
    bad[7] = n
    rc, msg = create(ptr, bad)
    assert rc == pg.ERR_ARG and "column index" in msg
    bad = idx.copy()
    bad[3] = -1
    assert create(ptr, bad)[0] == pg.ERR_ARG
    badp = ptr.copy()
    badp[10] = badp[11] + 1
    rc, msg = create(badp, idx)
    assert rc == pg.ERR_ARG and "monotone" in msg
    assert create(ptr, idx)[0] == 0  # the library is still usable


def test_bad_operator_handle_is_an_error():
    A = np.ones((5, 4))
    op = pg.CsrOperator(A)
    op.close()
    with pytest.raises(pg.PropackError):
        pg.svdp(op, 2, rng=rng0())


# ----------------------------------------------------- mixed form (FP32 + FP64 refinement)
MIXED_SIG_RTOL = 1e-10   # after the FP64 refinement: the FP64 bar
MIXED_VEC_TOL = 1e-8


@pytest.mark.parametrize("opts", [dict(), dict(cgs=True), dict(delta=-1.0, eta=-1.0)],
                         ids=["default", "cgs", "propack_defaults"])
def test_mixed_vs_golden(golden, opts):
    S, L, R = csr_from(golden, "lr_S"), csr_from(golden, "lr_L"), csr_from(golden, "lr_R")
    op = pg.CsrOperator(S, L, R, golden["lr_w"])
    u, s, vt, bnd = pg.svdp(op, 10, irl_mode=True, kmax=30, tol=1e-10, rng=rng0(), precision="mixed", **opts)
    st = pg.get_stats()
    assert st["nopx_low"] > 0, "the FP32 phase did not run"
    assert pg.get_precision() == "fp64"
    np.testing.assert_allclose(s, golden["lowrank_irl_sigma"], rtol=MIXED_SIG_RTOL)
    np.testing.assert_allclose(s, golden["lowrank_dense_sigma"][:10], rtol=MIXED_SIG_RTOL)
    uo = golden["lowrank_irl_u"] if "lowrank_irl_u" in golden else None
    res = max(max(np.linalg.norm(op.matvec(vt[i]) - s[i] * u[:, i]),
                  np.linalg.norm(op.rmatvec(u[:, i]) - s[i] * vt[i])) for i in range(10))
    assert res <= 1e-8 * s[0], res
    if uo is not None:
        assert subspace_err(u, uo) < MIXED_VEC_TOL
    op.close()


def test_mixed_plain_config0(golden):
    A = csr_from(golden, "plain")
    u, s, vt, bnd = pg.svdp(A, 10, irl_mode=True, kmax=40, tol=1e-12, rng=rng0(), precision="mixed")
    np.testing.assert_allclose(s, golden["plain_dense_sigma"][:10], rtol=1e-11)
    assert subspace_err(u, golden["plain_lansvd_u"]) < MIXED_VEC_TOL
    assert subspace_err(vt.T, golden["plain_lansvd_vt"].T) < MIXED_VEC_TOL


def test_mixed_host_callback(golden):
    M = csr_from(golden, "small").toarray()
    u, s, vt, bnd = pg.svdp(aslinearoperator(M), 3, tol=1e-8, rng=rng0(), precision="mixed")
    np.testing.assert_allclose(s, golden["small_irl_lm_sigma"], rtol=1e-8, atol=1e-8)


# ------------------------------------------------- Ritz vectors to the host
@pytest.mark.parametrize("driver", ["irl", "irl_complex", "plain", "irl_mixed"])
def test_ritz_vectors_into_page_locked_arrays(driver):
    """Above 2^20 rows the drivers form the Ritz vectors in row chunks and
    copy each chunk into a page-locked U, V while the next chunk is formed;
    the caller gets the same bits as through ordinary arrays (one product
    and one copy), and the values of the oracle (the mixed form: its FP64
    refinement's products)."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    m, n, k = 1_200_000, 2_000, 4
    cols = (rng.integers(0, n - 3, m)[:, None] + np.arange(3)).ravel()
    vals = rng.standard_normal(3 * m) * (1.0 + cols) ** -0.5
    cplx = driver == "irl_complex"
    if cplx:
        vals = vals * (1 + 0.5j)
    S = sp.csr_array((vals, cols, np.arange(0, 3 * m + 1, 3)), shape=(m, n))
    op = pg.CsrOperator(S)
    dt, tdt = (np.complex128, torch.complex128) if cplx else (np.float64, torch.float64)
    dim = 16 if driver != "plain" else 40
    u0 = np.random.default_rng(0).uniform(size=m)
    eps = np.finfo(np.float64).eps
    ioption = np.array([0, 1], dtype=np.int32)
    outs = []
    for pinned in (False, True):
        if pinned:
            U = torch.zeros((dim + 1, m), dtype=tdt).pin_memory().numpy().T
            V = torch.zeros((dim, n), dtype=tdt).pin_memory().numpy().T
        else:
            U = np.zeros((m, dim + 1), dtype=dt, order="F")
            V = np.zeros((n, dim), dtype=dt, order="F")
        U[:, 0] = u0
        sig, bnd = np.zeros(k), np.zeros(k)
        if driver == "plain":
            doption = np.array([np.sqrt(eps), eps ** 0.75, 0.0])
            nc, info = pg.lansvd(b"Y", b"Y", m, n, k, dim, op.aprod, U, sig, bnd, V, 1e-8, doption, ioption,
                                 iparm=op.iparm)
        else:
            doption = np.array([np.sqrt(eps), eps ** 0.75, 0.0, 0.002])
            call = pg.zlansvd_irl if cplx else pg.lansvd_irl
            if driver == "irl_mixed":
                pg.set_precision("mixed")
            try:
                nc, info = call(b"L", b"Y", b"Y", m, n, dim, dim - k, k, 30, op.aprod, U, sig, bnd, V, 1e-8,
                                doption, ioption, iparm=op.iparm)
            finally:
                pg.set_precision("fp64")
            if driver == "irl_mixed":
                assert pg.get_stats()["nopx_low"] > 0, "the FP32 phase did not run"
        assert info == 0 and nc == k
        outs.append((sig.copy(), np.array(U[:, :k]), np.array(V[:, :k])))
        del U, V
    op.close()
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    # no misplaced rows: every chunk's vectors satisfy A v = sigma u
    sig, Uk, Vk = outs[1]
    for i in range(k):
        r = S @ Vk[:, i] - sig[i] * Uk[:, i]
        assert np.linalg.norm(r) <= 1e-7 * sig[0], (i, np.linalg.norm(r))
    ref = oracle.svdp(S, k, irl_mode=driver != "plain", kmax=dim, tol=1e-8, v0=u0, maxiter=30)[1]
    np.testing.assert_allclose(outs[1][0], ref, rtol=MIXED_SIG_RTOL if driver == "irl_mixed" else SIG_RTOL)
