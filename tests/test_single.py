"""The single-precision drivers slansvd_ / slansvd_irl_ (REAL argument
lists of single/slansvd.F and single/slansvd_irl.F) through the C ABI, with
the device operator and with a user REAL APROD, against dense LAPACK.
FP32 tolerances: singular values 1e-5 relative, residuals 1e-5 * sigma_1."""
import ctypes as C

import numpy as np
import pytest

import propack_gb300 as pg
from conftest import csr_from

pytestmark = pytest.mark.gpu

SAPROD = C.CFUNCTYPE(None, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float),
                     C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_int), C.c_size_t)
fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
ipt = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
ci = lambda v: C.byref(C.c_int(v))


def _call(irl, A, k, kmax, aprod, iparm, tol=1e-5):
    L = pg.load()
    m, n = A.shape
    U = np.zeros((m, kmax + 1), dtype=np.float32, order="F")
    V = np.zeros((n, kmax), dtype=np.float32, order="F")
    U[:, 0] = np.random.default_rng(0).uniform(size=m)
    sig = np.zeros(k, dtype=np.float32)
    bnd = np.zeros(k, dtype=np.float32)
    lwork, liwork, _ = pg.work_sizes(m, n, kmax, irl=irl)
    work = np.empty(lwork, dtype=np.float32)
    iwork = np.empty(liwork, dtype=np.int32)
    dop = np.array([np.sqrt(np.finfo(np.float32).eps), np.finfo(np.float32).eps ** 0.75, 0.0, 0.002],
                   dtype=np.float32)
    iop = np.array([0, 1], dtype=np.int32)
    info = C.c_int(0)
    sparm = np.zeros(1, dtype=np.float32)
    if irl:
        ne = C.c_int(k)
        L.slansvd_irl_(b"L", b"y", b"y", ci(m), ci(n), ci(kmax), ci(kmax - k), C.byref(ne), ci(200), aprod, fp(U),
                       ci(m), fp(sig), fp(bnd), fp(V), ci(n), C.byref(C.c_float(tol)), fp(work), ci(lwork), ipt(iwork),
                       ci(liwork), fp(dop), ipt(iop), C.byref(info), fp(sparm), ipt(iparm), C.c_size_t(1),
                       C.c_size_t(1), C.c_size_t(1))
        kc = ne.value
    else:
        kk = C.c_int(k)
        L.slansvd_(b"y", b"y", ci(m), ci(n), C.byref(kk), ci(kmax), aprod, fp(U), ci(m), fp(sig), fp(bnd), fp(V),
                   ci(n), C.byref(C.c_float(tol)), fp(work), ci(lwork), ipt(iwork), ci(liwork), fp(dop), ipt(iop),
                   C.byref(info), fp(sparm), ipt(iparm), C.c_size_t(1), C.c_size_t(1))
        kc = kk.value
    return info.value, kc, sig, U[:, :k].astype(np.float64), V[:, :k].astype(np.float64)


def _check(A, info, kc, sig, U, V, k):
    assert info == 0 and kc == k
    Ad = A.toarray()
    sd = np.linalg.svd(Ad, compute_uv=False)[:k]
    np.testing.assert_allclose(sig, sd, rtol=1e-5)
    res = max(np.linalg.norm(Ad @ V[:, i] - sig[i] * U[:, i]) for i in range(k))
    assert res < 1e-5 * sd[0]


@pytest.mark.parametrize("irl", [True, False])
def test_single_precision_device_operator(golden, irl):
    A = csr_from(golden, "plain").astype(np.float32).astype(np.float64)
    op = pg.CsrOperator(A)
    aprod = C.cast(pg.load().propack_gpu_csr_saprod_, SAPROD)
    info, kc, sig, U, V = _call(irl, A, 10, 40 if irl else 200, aprod, op.iparm)
    _check(A, info, kc, sig, U, V, 10)
    op.close()


def test_single_precision_user_aprod(golden):
    A = csr_from(golden, "plain").astype(np.float32).astype(np.float64)
    A32 = A.astype(np.float32)
    m, n = A.shape

    def cb(transa, pm, pn, px, py, sparm, iparm, ln):
        if transa[0:1].lower() == b"t":
            x = np.ctypeslib.as_array(px, shape=(m,))
            np.ctypeslib.as_array(py, shape=(n,))[:] = A32.T @ x
        else:
            x = np.ctypeslib.as_array(px, shape=(n,))
            np.ctypeslib.as_array(py, shape=(m,))[:] = A32 @ x
    aprod = SAPROD(cb)
    info, kc, sig, U, V = _call(True, A, 6, 30, aprod, np.zeros(2, dtype=np.int32))
    _check(A, info, kc, sig, U, V, 6)
