"""Oracle harness: ctypes access to propack_oracle.c.

TEST INFRASTRUCTURE ONLY -- the oracle of the GPU library's tests and the timed
CPU baseline of bench.py.  The product (propack_gb300/) never imports this.

The entry points take the reference's Fortran argument lists
(double/dlansvd.F:1-3, double/dlansvd_irl.F:1-3) through the same
gfortran calling convention as the GPU library's C ABI, so one harness
(`call_lansvd`, `call_lansvd_irl`) drives either library.
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle_propack.so")
SRC = os.path.join(_HERE, "propack_oracle.c")
SRC_Z = os.path.join(_HERE, "propack_oracle_z.inc")

APROD = C.CFUNCTYPE(None, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                    C.POINTER(C.c_double), C.POINTER(C.c_double),
                    C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_size_t)

_lib = None


def build(force=False):
    """Compile the oracle with gcc + OpenMP into oracle/_build/."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(SRC), os.path.getmtime(SRC_Z))):
        return LIB_PATH
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", LIB_PATH, SRC, "-lm"]
    subprocess.check_call(cmd)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        i64p = C.POINTER(C.c_int64)
        L.oracle_op_create.restype = C.c_void_p
        L.oracle_op_create.argtypes = [C.c_int, C.c_int, i64p, ip, dp, C.c_int,
                                       i64p, ip, dp, i64p, ip, dp, dp]
        L.oracle_op_destroy.argtypes = [C.c_void_p]
        L.oracle_bdsqr.argtypes = [C.c_int, dp, dp, C.c_int, dp, C.c_int, C.c_int, dp, C.c_int]
        L.oracle_bdsqr.restype = C.c_int
        L.oracle_getstat.argtypes = [C.POINTER(C.c_long)]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_lanbpro_sample.restype = C.c_int
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Operator:
    """A = S + L diag(w) R^T held by the oracle; S, L, R scipy CSR."""

    def __init__(self, S, L=None, R=None, w=None):
        import scipy.sparse as sp
        # copy: sorting the indices of a view would permute the caller's data
        S = sp.csr_array(S, dtype=np.float64, copy=True)
        S.sort_indices()
        self.shape = S.shape
        self._keep = []

        def parts(M):
            M = sp.csr_array(M, dtype=np.float64)
            ptr = np.ascontiguousarray(M.indptr, dtype=np.int64)
            idx = np.ascontiguousarray(M.indices, dtype=np.int32)
            val = np.ascontiguousarray(M.data, dtype=np.float64)
            self._keep += [ptr, idx, val]
            return (ptr.ctypes.data_as(C.POINTER(C.c_int64)), _ip(idx), _dp(val))

        r = 0 if L is None else L.shape[1]
        sp_ = parts(S)
        if r:
            lp, rp = parts(L), parts(R)
            w = np.ascontiguousarray(w, dtype=np.float64)
            self._keep.append(w)
            wp = _dp(w)
        else:
            null64 = C.POINTER(C.c_int64)()
            lp = rp = (null64, C.POINTER(C.c_int)(), C.POINTER(C.c_double)())
            wp = C.POINTER(C.c_double)()
        self.handle = lib().oracle_op_create(S.shape[0], S.shape[1], *sp_, r, *lp, *rp, wp)
        h = int(self.handle)
        self.iparm = np.array([h & 0xFFFFFFFF, (h >> 32) & 0xFFFFFFFF], dtype=np.uint32).view(np.int32)
        self.aprod = C.cast(lib().oracle_op_aprod, APROD)

    def __del__(self):
        try:
            lib().oracle_op_destroy(C.c_void_p(self.handle))
        except Exception:
            pass


def python_aprod(A):
    """An APROD callback (gfortran convention) over any object with
    matvec/rmatvec or a dense/sparse matrix."""
    from scipy.sparse.linalg import aslinearoperator
    op = aslinearoperator(A)
    m, n = op.shape

    def cb(transa, pm, pn, px, py, dparm, iparm, ln):
        t = transa[0:1].lower() == b't'
        if t:
            x = np.ctypeslib.as_array(px, shape=(m,))
            y = np.ctypeslib.as_array(py, shape=(n,))
            y[:] = op.rmatvec(x)
        else:
            x = np.ctypeslib.as_array(px, shape=(n,))
            y = np.ctypeslib.as_array(py, shape=(m,))
            y[:] = op.matvec(x)
    return APROD(cb)


def call_lansvd(fn, jobu, jobv, m, n, k, kmax, aprod, U, sigma, bnd, V, tol, doption, ioption,
                iparm=None, dparm=None, lwork=None, liwork=None):
    """Invoke a dlansvd_-shaped entry point; returns (k_converged, info)."""
    ci = lambda v: C.byref(C.c_int(v))
    km = C.c_int(k)
    info = C.c_int(0)
    if lwork is None:
        lwork = m + n + 9 * kmax + 5 * kmax ** 2 + 4 + max(3 * kmax ** 2 + 4 * kmax + 4, 32 * max(m, n))
    if liwork is None:
        liwork = 8 * kmax
    work = np.zeros(max(lwork, 1))
    iwork = np.zeros(max(liwork, 1), dtype=np.int32)
    iparm = np.zeros(2, dtype=np.int32) if iparm is None else iparm
    dparm = np.zeros(1) if dparm is None else dparm
    tolc = C.c_double(tol)
    fn(jobu, jobv, ci(m), ci(n), C.byref(km), ci(kmax), aprod, _dp(U), ci(U.shape[0]),
       _dp(sigma), _dp(bnd), _dp(V), ci(V.shape[0]), C.byref(tolc), _dp(work), ci(lwork),
       _ip(iwork), ci(liwork), _dp(doption), _ip(ioption), C.byref(info), _dp(dparm), _ip(iparm),
       C.c_size_t(1), C.c_size_t(1))
    return km.value, info.value


def call_lansvd_irl(fn, which, jobu, jobv, m, n, dim, p, neig, maxiter, aprod, U, sigma, bnd, V, tol,
                    doption, ioption, iparm=None, dparm=None, lwork=None, liwork=None):
    """Invoke a dlansvd_irl_-shaped entry point; returns (neig_converged, info)."""
    ci = lambda v: C.byref(C.c_int(v))
    ne = C.c_int(neig)
    info = C.c_int(0)
    if lwork is None:
        lwork = m + n + 10 * dim + 5 * dim ** 2 + 4 + max(3 * dim ** 2 + 4 * dim + 4, 32 * max(m, n))
    if liwork is None:
        liwork = 8 * dim
    work = np.zeros(max(lwork, 1))
    iwork = np.zeros(max(liwork, 1), dtype=np.int32)
    iparm = np.zeros(2, dtype=np.int32) if iparm is None else iparm
    dparm = np.zeros(1) if dparm is None else dparm
    tolc = C.c_double(tol)
    fn(which, jobu, jobv, ci(m), ci(n), ci(dim), ci(p), C.byref(ne), ci(maxiter), aprod, _dp(U),
       ci(U.shape[0]), _dp(sigma), _dp(bnd), _dp(V), ci(V.shape[0]), C.byref(tolc), _dp(work),
       ci(lwork), _ip(iwork), ci(liwork), _dp(doption), _ip(ioption), C.byref(info), _dp(dparm),
       _ip(iparm), C.c_size_t(1), C.c_size_t(1), C.c_size_t(1))
    return ne.value, info.value


def getstat():
    out = (C.c_long * 8)()
    lib().oracle_getstat(out)
    keys = ("nopx", "nreorth", "ndot", "nitref", "nbsvd", "nrestart", "nlandim", "nsing")
    return dict(zip(keys, list(out)))


def clearstat():
    lib().oracle_clearstat()


def nelr():
    """Passes of the extended local reorthogonalisation since clearstat()."""
    L = lib()
    L.oracle_nelr.restype = C.c_long
    return int(L.oracle_nelr())


def bdsqr(d, e, nru_vectors=False, ncvt_vectors=False, urow=None):
    """Upper-bidiagonal SVD of the oracle (for pinning against numpy)."""
    n = len(d)
    d = np.array(d, dtype=np.float64)
    e = np.array(list(e) + [0.0], dtype=np.float64)
    if nru_vectors:
        U = np.asfortranarray(np.eye(n))
        nru, ldu = n, n
    elif urow is not None:
        U = np.asfortranarray(np.array(urow, dtype=np.float64).reshape(1, n))
        nru, ldu = 1, 1
    else:
        U = np.zeros((1, 1))
        nru, ldu = 0, 1
    if ncvt_vectors:
        VT = np.asfortranarray(np.eye(n))
        ncvt = n
    else:
        VT = np.zeros((1, 1))
        ncvt = 0
    info = lib().oracle_bdsqr(n, _dp(d), _dp(e), ncvt, _dp(VT), max(n, 1), nru, _dp(U), ldu)
    return d, U, VT, info


def svdp(A, k, which='LM', irl_mode=True, kmax=None, compute_u=True, compute_v=True, v0=None,
         tol=0, delta=None, eta=None, anorm=0, cgs=False, elr=True, min_relgap=0.002, shifts=None,
         maxiter=None, rng=None, op=None):
    """The oracle behind scipy's `_svdp` argument conventions
    (scipy/sparse/linalg/_svdp.py): same defaults, same start vector
    u[:, 0] = rng.uniform(size=m).  Returns (u, sigma, vt, bnd, info, k_conv)."""
    L = lib()
    if op is None and not callable(getattr(A, "matvec", None)):
        op = ZOperator(A) if np.iscomplexobj(A.data if hasattr(A, "data") else A) else Operator(A)
    if isinstance(op, ZOperator):
        return _zsvdp(op, k, which, irl_mode, kmax, compute_u, compute_v, v0, tol, delta, eta, anorm, cgs, elr,
                      min_relgap, shifts, maxiter, rng)
    m, n = (op.shape if op is not None else A.shape)
    if kmax is None:
        kmax = 10 * k
    if maxiter is None:
        maxiter = 1000
    kmax = min(m + 1, n + 1, kmax)
    u = np.zeros((m, kmax + 1), order='F')
    v = np.zeros((n, kmax), order='F')
    sigma = np.zeros(k)
    bnd = np.zeros(k)
    if v0 is None:
        u[:, 0] = rng.uniform(size=m)
    else:
        u[:, 0] = v0
    if delta is None:
        delta = np.sqrt(np.finfo(np.float64).eps)
    if eta is None:
        eta = np.finfo(np.float64).eps ** 0.75
    ioption = np.array([int(bool(cgs)), int(bool(elr))], dtype=np.int32)
    if op is not None:
        aprod, iparm = op.aprod, op.iparm
    else:
        aprod, iparm = python_aprod(A), None
    jobu = b'y' if compute_u else b'n'
    jobv = b'y' if compute_v else b'n'
    if irl_mode:
        doption = np.array([delta, eta, anorm, min_relgap], dtype=np.float64)
        if shifts is None:
            shifts = kmax - k
        kc, info = call_lansvd_irl(L.oracle_dlansvd_irl, b'L' if which == 'LM' else b'S', jobu, jobv,
                                   m, n, kmax, shifts, k, maxiter, aprod, u, sigma, bnd, v, tol,
                                   doption, ioption, iparm=iparm)
    else:
        doption = np.array([delta, eta, anorm], dtype=np.float64)
        kc, info = call_lansvd(L.oracle_dlansvd, jobu, jobv, m, n, k, kmax, aprod, u, sigma, bnd, v,
                               tol, doption, ioption, iparm=iparm)
    return u[:, :k], sigma, v[:, :k].T, bnd, info, kc


# ------------------------------------------------------------------ complex
ZAPROD = C.CFUNCTYPE(None, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p, C.c_void_p,
                     C.c_void_p, C.POINTER(C.c_int), C.c_size_t)


def _vp(a):
    return C.c_void_p(a.ctypes.data)


class ZOperator:
    """Complex A (m x n, scipy CSR) held by the oracle with A^H built once;
    its APROD serves TRANSA 'n' (A x) and 'c' (A^H x), as
    complex16/zlanbpro.F calls it."""

    def __init__(self, A):
        import scipy.sparse as sp
        A = sp.csr_array(A, dtype=np.complex128, copy=True)
        A.sort_indices()
        self.shape = A.shape
        self._keep = [np.ascontiguousarray(A.indptr, dtype=np.int64), np.ascontiguousarray(A.indices, dtype=np.int32),
                      np.ascontiguousarray(A.data, dtype=np.complex128)]
        L = lib()
        L.oracle_zop_create.restype = C.c_void_p
        L.oracle_zop_create.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_zop_destroy.argtypes = [C.c_void_p]
        self.handle = L.oracle_zop_create(A.shape[0], A.shape[1], *(_vp(a) for a in self._keep))
        h = int(self.handle)
        self.iparm = np.array([h & 0xFFFFFFFF, (h >> 32) & 0xFFFFFFFF], dtype=np.uint32).view(np.int32)
        self.aprod = C.cast(L.oracle_zop_aprod, ZAPROD)

    def __del__(self):
        try:
            lib().oracle_zop_destroy(C.c_void_p(self.handle))
        except Exception:
            pass


def _zsvdp(op, k, which, irl_mode, kmax, compute_u, compute_v, v0, tol, delta, eta, anorm, cgs, elr,
           min_relgap, shifts, maxiter, rng):
    """The complex path of svdp: scipy's _svdp conventions for complex input
    (start vector uniform + 1j*uniform, zlansvd / zlansvd_irl)."""
    L = lib()
    m, n = op.shape
    if kmax is None:
        kmax = 10 * k
    if maxiter is None:
        maxiter = 1000
    kmax = min(m + 1, n + 1, kmax)
    u = np.zeros((m, kmax + 1), order='F', dtype=np.complex128)
    v = np.zeros((n, kmax), order='F', dtype=np.complex128)
    sigma = np.zeros(k)
    bnd = np.zeros(k)
    if v0 is None:
        u[:, 0] = rng.uniform(size=m)
        u[:, 0] += 1j * rng.uniform(size=m)
    else:
        u[:, 0] = v0
    if delta is None:
        delta = np.sqrt(np.finfo(np.float64).eps)
    if eta is None:
        eta = np.finfo(np.float64).eps ** 0.75
    ioption = np.array([int(bool(cgs)), int(bool(elr))], dtype=np.int32)
    jobu = b'y' if compute_u else b'n'
    jobv = b'y' if compute_v else b'n'
    ci = lambda x: C.byref(C.c_int(x))
    lwork = m + n + 10 * kmax + 5 * kmax ** 2 + 4 + max(3 * kmax ** 2 + 4 * kmax + 4, 32 * max(m, n))
    work = np.zeros(lwork)
    zwork = np.zeros(m + n + kmax, dtype=np.complex128)
    iwork = np.zeros(8 * kmax + 8, dtype=np.int32)
    zparm = np.zeros(1, dtype=np.complex128)
    info = C.c_int(0)
    tolc = C.c_double(tol)
    if irl_mode:
        doption = np.array([delta, eta, anorm, min_relgap], dtype=np.float64)
        if shifts is None:
            shifts = kmax - k
        ne = C.c_int(k)
        L.oracle_zlansvd_irl(b'L' if which == 'LM' else b'S', jobu, jobv, ci(m), ci(n), ci(kmax), ci(shifts),
                             C.byref(ne), ci(maxiter), op.aprod, _vp(u), ci(m), _dp(sigma), _dp(bnd), _vp(v), ci(n),
                             C.byref(tolc), _dp(work), ci(lwork), _vp(zwork), ci(zwork.size), _ip(iwork),
                             ci(iwork.size), _dp(doption), _ip(ioption), C.byref(info), _vp(zparm), _ip(op.iparm),
                             C.c_size_t(1), C.c_size_t(1), C.c_size_t(1))
    else:
        doption = np.array([delta, eta, anorm], dtype=np.float64)
        ne = C.c_int(k)
        L.oracle_zlansvd(jobu, jobv, ci(m), ci(n), C.byref(ne), ci(kmax), op.aprod, _vp(u), ci(m), _dp(sigma),
                         _dp(bnd), _vp(v), ci(n), C.byref(tolc), _dp(work), ci(lwork), _vp(zwork), ci(zwork.size),
                         _ip(iwork), ci(iwork.size), _dp(doption), _ip(ioption), C.byref(info), _vp(zparm),
                         _ip(op.iparm), C.c_size_t(1), C.c_size_t(1))
    return u[:, :k], sigma, v[:, :k].conj().T, bnd, info.value, ne.value
