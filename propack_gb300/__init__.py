"""propack_gb300 -- GB300-native Lanczos bidiagonalisation (PROPACK's hot path).

The product is the C-ABI library ``_lib/libpropack_gb300.so`` (CUDA, sm_103a);
this module is the thin Python host side over it:

* ``svdp`` mirrors scipy's PROPACK front end (scipy/sparse/linalg/_svdp.py,
  ``_svdp``): same arguments, defaults, start vector and return values, but
  every call runs the GPU drivers ``dlansvd_irl_`` / ``dlansvd_`` through the
  C ABI.
* Complex matrices go to the complex*16 drivers ``zlansvd_irl_`` /
  ``zlansvd_`` the same way.
* ``CsrOperator`` uploads A = S + L diag(w) R' to the device; passing it (or
  a scipy sparse / dense matrix, which is wrapped automatically) makes the
  drivers use the device operator with no host round trips.  A
  LinearOperator is called back on the host through the reference's APROD
  convention.

There is no CPU fallback: if the library is missing or no CUDA device is
usable, the calls raise.
"""
import ctypes as C
import os

import numpy as np

from . import _build

__all__ = ["svdp", "CsrOperator", "load", "get_stats", "clearstat", "printstat", "PropackError", "APROD", "ZAPROD"]

APROD = C.CFUNCTYPE(None, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                    C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_size_t)
# the complex*16 APROD of complex16/zlanbpro.F (x, y, zparm: complex*16 arrays)
ZAPROD = C.CFUNCTYPE(None, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p, C.c_void_p,
                     C.c_void_p, C.POINTER(C.c_int), C.c_size_t)

ERR_ARG, ERR_CUDA, ERR_HANDLE, ERR_WAIT = -2, -3, -4, -5


class PropackError(RuntimeError):
    pass


class _Stats(C.Structure):
    _fields_ = [("nopx", C.c_int64), ("nreorth", C.c_int64), ("ndot", C.c_int64), ("nrestart", C.c_int64),
                ("nbsvd", C.c_int64), ("nlandim", C.c_int64), ("device_ms", C.c_double),
                ("lanczos_ms", C.c_double), ("bsvd_ms", C.c_double), ("gemm_ms", C.c_double),
                ("kernel_launches", C.c_int64), ("solve_ms", C.c_double), ("nopx_low", C.c_int64),
                ("low_ms", C.c_double), ("cgs_cols_u", C.c_int64), ("cgs_cols_v", C.c_int64)]


PROFILE_KINDS = ("spmv_adj", "spmv_fwd", "elr", "cgs_dots", "cgs_upd", "lowrank_prepass", "analyse", "sweeps",
                 "gemm", "spmv_adj_fp32", "spmv_fwd_fp32", "cgs_dots_fp32", "cgs_upd_fp32", "ritz_prep")


_lib = None


def load(build_if_missing=True):
    """Load libpropack_gb300.so (building it in-tree if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB) or not _build.up_to_date():
        if not build_if_missing:
            raise PropackError(f"{_build.LIB} is not built")
        _build.build()
    L = C.CDLL(_build.LIB)
    dp, ip, i64p = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_int64)
    L.propack_csr_create.restype = C.c_int
    L.propack_csr_create.argtypes = [C.c_int, C.c_int, i64p, ip, dp, C.c_int, i64p, ip, dp, i64p, ip, dp, dp, i64p]
    L.propack_csr_destroy.restype = C.c_int
    L.propack_csr_destroy.argtypes = [C.c_int64]
    L.propack_zcsr_create.restype = C.c_int
    L.propack_zcsr_create.argtypes = [C.c_int, C.c_int, i64p, ip, C.c_void_p, i64p]
    L.propack_zcsr_expand.restype = C.c_int
    L.propack_zcsr_expand.argtypes = [C.c_int, C.c_int, i64p, ip, C.c_void_p, i64p, ip, dp]
    L.propack_set_zcsr_form.restype = C.c_int
    L.propack_set_zcsr_form.argtypes = [C.c_int]
    L.propack_last_error.restype = C.c_char_p
    L.propack_get_stats.argtypes = [C.POINTER(_Stats)]
    _lib = L
    return L


def last_error():
    return load().propack_last_error().decode(errors="replace")


def get_stats():
    s = _Stats()
    load().propack_get_stats(C.byref(s))
    return {k: getattr(s, k) for k, _ in _Stats._fields_}


def clearstat():
    load().clearstat_()


def set_profiling(on):
    load().propack_set_profiling(1 if on else 0)


def get_profile():
    """{kernel class: (launches, total ms)} since set_profiling(True)."""
    L = load()
    n = len(PROFILE_KINDS)
    ms = (C.c_double * n)()
    cnt = (C.c_int64 * n)()
    L.propack_get_profile(ms, cnt, n)
    return {k: (int(cnt[i]), float(ms[i])) for i, k in enumerate(PROFILE_KINDS)}


def set_spmv_schedule(mode):
    """SpMV schedule of operators built afterwards: "rule" (default: chunked
    below 128 nonzeros per row), "chunked", "staged" or "tuned" (timed on
    the device; propack_set_spmv_schedule)."""
    m = {"rule": 0, "chunked": 1, "staged": 2, "tuned": 3}[mode]
    if load().propack_set_spmv_schedule(m) != 0:
        raise PropackError("propack_set_spmv_schedule failed")


def printstat():
    load().printstat_()


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _i64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64))


class CsrOperator:
    """Device-resident A = S + L diag(w) R' (S: m x n, L: m x r, R: n x r).

    S, L, R are anything scipy.sparse.csr_array accepts.  The transposed
    operator is built on the device.  ``iparm`` is the two-int array that
    carries the handle through the reference's APROD argument list."""

    def __init__(self, S, L=None, R=None, w=None):
        import scipy.sparse as sp
        lib = load()
        S = sp.csr_array(S)
        self.shape = S.shape
        if np.iscomplexobj(S.data):
            self._init_complex(lib, S, L)
            return
        self.dtype = np.dtype(np.float64)
        keep = []

        def parts(M):
            M = sp.csr_array(M)
            ptr = np.ascontiguousarray(M.indptr, dtype=np.int64)
            idx = np.ascontiguousarray(M.indices, dtype=np.int32)
            val = np.ascontiguousarray(M.data, dtype=np.float64)
            keep.extend([ptr, idx, val])
            return _i64p(ptr), _ip(idx), _dp(val)

        r = 0 if L is None else int(L.shape[1])
        sp_ = parts(S)
        if r:
            lp, rp = parts(L), parts(R)
            w = np.ascontiguousarray(w, dtype=np.float64)
            keep.append(w)
            wp = _dp(w)
        else:
            lp = rp = (C.POINTER(C.c_int64)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)())
            wp = C.POINTER(C.c_double)()
        h = C.c_int64(0)
        rc = lib.propack_csr_create(S.shape[0], S.shape[1], *sp_, r, *lp, *rp, wp, C.byref(h))
        if rc != 0:
            raise PropackError(f"propack_csr_create failed ({rc}): {last_error()}")
        self.handle = h.value
        self.iparm = np.array([h.value & 0xFFFFFFFF, (h.value >> 32) & 0xFFFFFFFF], dtype=np.uint32).view(np.int32)
        self.aprod = C.cast(lib.propack_gpu_csr_aprod_, APROD)
        self.r = r

    def _init_complex(self, lib, S, L):
        # a complex S alone (propack_zcsr_create): the device holds it as a
        # native complex CSR (or its real 2x2-block form, set_complex_form),
        # which the complex drivers apply as A and A^H
        if L is not None:
            raise TypeError("a complex operator takes no low-rank term")
        self.dtype = np.dtype(np.complex128)
        ptr = np.ascontiguousarray(S.indptr, dtype=np.int64)
        idx = np.ascontiguousarray(S.indices, dtype=np.int32)
        val = np.ascontiguousarray(S.data, dtype=np.complex128)
        h = C.c_int64(0)
        rc = lib.propack_zcsr_create(S.shape[0], S.shape[1], _i64p(ptr), _ip(idx), C.c_void_p(val.ctypes.data),
                                     C.byref(h))
        if rc != 0:
            raise PropackError(f"propack_zcsr_create failed ({rc}): {last_error()}")
        self.handle = h.value
        self.iparm = np.array([h.value & 0xFFFFFFFF, (h.value >> 32) & 0xFFFFFFFF], dtype=np.uint32).view(np.int32)
        self.aprod = C.cast(lib.propack_gpu_csr_zaprod_, ZAPROD)
        self.r = 0

    @property
    def schedule(self):
        """({'fwd': ..., 'adj': ...} with 'chunked' / 'staged', timed ms per
        product {(direction, schedule): ms} where the choice was timed)."""
        sched = (C.c_int * 2)()
        ms = (C.c_float * 4)()
        rc = load().propack_csr_schedule(C.c_int64(self.handle), sched, ms)
        if rc != 0:
            raise PropackError(f"propack_csr_schedule failed ({rc})")
        names = {1: "chunked", 0: "staged"}
        timed = {(d, s_): ms[2 * i + j] for i, d in enumerate(("fwd", "adj"))
                 for j, s_ in enumerate(("chunked", "staged")) if ms[2 * i + j] > 0}
        return {"fwd": names[sched[0]], "adj": names[sched[1]]}, timed

    def close(self):
        if getattr(self, "handle", 0):
            load().propack_csr_destroy(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _apply(self, trans, x):
        m, n = self.shape
        ci = lambda v: C.byref(C.c_int(v))
        if self.dtype == np.complex128:
            x = np.ascontiguousarray(x, dtype=np.complex128)
            y = np.zeros(n if trans else m, dtype=np.complex128)
            load().propack_gpu_csr_zaprod_(b'c' if trans else b'n', ci(m), ci(n), C.c_void_p(x.ctypes.data),
                                           C.c_void_p(y.ctypes.data), C.c_void_p(), _ip(self.iparm), C.c_size_t(1))
            return y
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(n if trans else m)
        ci = lambda v: C.byref(C.c_int(v))
        load().propack_gpu_csr_aprod_(b't' if trans else b'n', ci(m), ci(n), _dp(x), _dp(y),
                                      C.POINTER(C.c_double)(), _ip(self.iparm), C.c_size_t(1))
        return y

    def matvec(self, x):
        return self._apply(False, x)

    def rmatvec(self, x):
        return self._apply(True, x)


def _host_aprod(A):
    from scipy.sparse.linalg import aslinearoperator
    op = aslinearoperator(A)
    m, n = op.shape

    def cb(transa, pm, pn, px, py, dparm, iparm, ln):
        if transa[0:1].lower() == b't':
            x = np.ctypeslib.as_array(px, shape=(m,))
            np.ctypeslib.as_array(py, shape=(n,))[:] = op.rmatvec(x)
        else:
            x = np.ctypeslib.as_array(px, shape=(n,))
            np.ctypeslib.as_array(py, shape=(m,))[:] = op.matvec(x)
    return APROD(cb)


def _host_zaprod(A):
    """ZAPROD over a complex host operator: 'n' y = A x, 'c' y = A^H x."""
    from scipy.sparse.linalg import aslinearoperator
    op = aslinearoperator(A)
    m, n = op.shape

    def cb(transa, pm, pn, px, py, zparm, iparm, ln):
        if transa[0:1].lower() == b'n':
            x = np.ctypeslib.as_array(C.cast(px, C.POINTER(C.c_double)), shape=(2 * n,)).view(np.complex128)
            y = np.ctypeslib.as_array(C.cast(py, C.POINTER(C.c_double)), shape=(2 * m,)).view(np.complex128)
            y[:] = op.matvec(x)
        else:
            x = np.ctypeslib.as_array(C.cast(px, C.POINTER(C.c_double)), shape=(2 * m,)).view(np.complex128)
            y = np.ctypeslib.as_array(C.cast(py, C.POINTER(C.c_double)), shape=(2 * n,)).view(np.complex128)
            y[:] = op.rmatvec(x)
    return ZAPROD(cb)


def work_sizes(m, n, kmax, vectors=True, irl=True, cplx=False):
    """LWORK, LIWORK and (complex drivers) LZWRK as the reference documents
    them (double/dlansvd.F:55-65, double/dlansvd_irl.F:65-75, with the
    block size NB = 32 that scipy's _svdp uses).  The drivers here validate
    the declared sizes (they refuse less than the reference itself writes)
    but never read or write WORK, IWORK or ZWORK."""
    nb = 32
    if vectors:
        lwork = m + n + (10 if irl else 9) * kmax + 5 * kmax ** 2 + 4 + max(3 * kmax ** 2 + 4 * kmax + 4,
                                                                           nb * max(m, n))
        liwork = 8 * kmax
    else:
        lwork = m + n + (10 if irl else 9) * kmax + 2 * kmax ** 2 + (5 if irl else 4) + max(m + n, 4 * kmax + 4)
        liwork = 2 * kmax + 2
    return lwork, liwork, (m + n + kmax if cplx else 0)


def _workspace(m, n, kmax, irl, cplx=False, dtype=np.float64):
    """Workspace arrays of the documented sizes (np.empty: never touched, so
    never paged in) and their sizes."""
    lwork, liwork, lzwrk = work_sizes(m, n, kmax, True, irl, cplx)
    return (np.empty(lwork, dtype=dtype), lwork, np.empty(liwork, dtype=np.int32), liwork,
            np.empty(max(lzwrk, 1), dtype=np.complex128), lzwrk)


def zlansvd_irl(which, jobu, jobv, m, n, dim, p, neig, maxiter, aprod, U, sigma, bnd, V, tol, doption, ioption,
                iparm=None):
    """Call zlansvd_irl_ with the reference's argument list (complex16/zlansvd_irl.F:1-3); U, V complex128
    Fortran-ordered.  Returns (neig_conv, info)."""
    lib = load()
    ci = lambda v: C.byref(C.c_int(v))
    ne, info = C.c_int(neig), C.c_int(0)
    work, lwork, iwork, liwork, zwork, lzwrk = _workspace(m, n, dim, True, True)
    zparm = np.zeros(1, dtype=np.complex128)
    iparm = np.zeros(2, dtype=np.int32) if iparm is None else iparm
    vp = lambda a: C.c_void_p(a.ctypes.data)
    lib.zlansvd_irl_(which, jobu, jobv, ci(m), ci(n), ci(dim), ci(p), C.byref(ne), ci(maxiter), aprod, vp(U),
                     ci(U.shape[0]), _dp(sigma), _dp(bnd), vp(V), ci(V.shape[0]), C.byref(C.c_double(tol)),
                     _dp(work), ci(lwork), vp(zwork), ci(lzwrk), _ip(iwork), ci(liwork), _dp(doption), _ip(ioption),
                     C.byref(info), vp(zparm), _ip(iparm), C.c_size_t(1), C.c_size_t(1), C.c_size_t(1))
    return ne.value, info.value


def zlansvd(jobu, jobv, m, n, k, kmax, aprod, U, sigma, bnd, V, tol, doption, ioption, iparm=None):
    """Call zlansvd_ with the reference's argument list (complex16/zlansvd.F:1-3).  Returns (k_conv, info)."""
    lib = load()
    ci = lambda v: C.byref(C.c_int(v))
    km, info = C.c_int(k), C.c_int(0)
    work, lwork, iwork, liwork, zwork, lzwrk = _workspace(m, n, kmax, False, True)
    zparm = np.zeros(1, dtype=np.complex128)
    iparm = np.zeros(2, dtype=np.int32) if iparm is None else iparm
    vp = lambda a: C.c_void_p(a.ctypes.data)
    lib.zlansvd_(jobu, jobv, ci(m), ci(n), C.byref(km), ci(kmax), aprod, vp(U), ci(U.shape[0]), _dp(sigma),
                 _dp(bnd), vp(V), ci(V.shape[0]), C.byref(C.c_double(tol)), _dp(work), ci(lwork), vp(zwork),
                 ci(lzwrk), _ip(iwork), ci(liwork), _dp(doption), _ip(ioption), C.byref(info), vp(zparm), _ip(iparm),
                 C.c_size_t(1), C.c_size_t(1))
    return km.value, info.value


def lansvd_irl(which, jobu, jobv, m, n, dim, p, neig, maxiter, aprod, U, sigma, bnd, V, tol, doption, ioption,
               iparm=None, dparm=None):
    """Call dlansvd_irl_ with the reference's argument list; returns (neig_conv, info)."""
    lib = load()
    ci = lambda v: C.byref(C.c_int(v))
    ne, info = C.c_int(neig), C.c_int(0)
    work, lwork, iwork, liwork, _, _ = _workspace(m, n, dim, True)
    iparm = np.zeros(2, dtype=np.int32) if iparm is None else iparm
    dparm = np.zeros(1) if dparm is None else dparm
    lib.dlansvd_irl_(which, jobu, jobv, ci(m), ci(n), ci(dim), ci(p), C.byref(ne), ci(maxiter), aprod, _dp(U),
                     ci(U.shape[0]), _dp(sigma), _dp(bnd), _dp(V), ci(V.shape[0]), C.byref(C.c_double(tol)),
                     _dp(work), ci(lwork), _ip(iwork), ci(liwork), _dp(doption), _ip(ioption), C.byref(info),
                     _dp(dparm), _ip(iparm), C.c_size_t(1), C.c_size_t(1), C.c_size_t(1))
    return ne.value, info.value


def lansvd(jobu, jobv, m, n, k, kmax, aprod, U, sigma, bnd, V, tol, doption, ioption, iparm=None, dparm=None):
    """Call dlansvd_ with the reference's argument list; returns (k_conv, info)."""
    lib = load()
    ci = lambda v: C.byref(C.c_int(v))
    km, info = C.c_int(k), C.c_int(0)
    work, lwork, iwork, liwork, _, _ = _workspace(m, n, kmax, False)
    iparm = np.zeros(2, dtype=np.int32) if iparm is None else iparm
    dparm = np.zeros(1) if dparm is None else dparm
    lib.dlansvd_(jobu, jobv, ci(m), ci(n), C.byref(km), ci(kmax), aprod, _dp(U), ci(U.shape[0]), _dp(sigma),
                 _dp(bnd), _dp(V), ci(V.shape[0]), C.byref(C.c_double(tol)), _dp(work), ci(lwork), _ip(iwork),
                 ci(liwork), _dp(doption), _ip(ioption), C.byref(info), _dp(dparm), _ip(iparm), C.c_size_t(1),
                 C.c_size_t(1))
    return km.value, info.value


_which_converter = {"LM": b"L", "SM": b"S"}


PRECISIONS = {"fp64": 0, "mixed": 1, "fp32": 2}


def set_precision(precision):
    """'fp64' (the reference's method) or 'mixed' (FP32 Lanczos vectors with
    FP64 scalars, then a short FP64 refinement) for this host thread."""
    rc = load().propack_set_precision(PRECISIONS[precision])
    if rc != 0:
        raise PropackError(f"propack_set_precision failed ({rc})")


def release_memory():
    """Return the device memory the library's pool keeps for reuse."""
    if load().propack_release_memory() != 0:
        raise PropackError(f"propack_release_memory failed: {last_error()}")


def set_cgs_arith(arith):
    """Gram-Schmidt arithmetic of the FP64 form for this host thread:
    "planes" (the default: each basis column split once into FP32 (hi, lo)
    planes, products summed on the FP32 pipe), "fp64" (FP64 FMAs) or "f3"
    (exact three-way FP32 splits of every element read; propack_set_cgs_arith)."""
    rc = load().propack_set_cgs_arith({"fp64": 0, "f3": 1, "planes": 2}[arith])
    if rc != 0:
        raise PropackError(f"propack_set_cgs_arith failed ({rc})")


def set_complex_form(form):
    """Form of complex device operators created afterwards (process-wide):
    "native" (the default: complex CSR, one index and one complex value per
    entry, complex SpMV) or "block" (the real 2x2-block form applied by the
    real kernels; propack_set_zcsr_form)."""
    rc = load().propack_set_zcsr_form({"native": 0, "block": 1}[form])
    if rc != 0:
        raise PropackError(f"propack_set_zcsr_form failed ({rc})")


def get_precision():
    mode = load().propack_get_precision()
    return {v: k for k, v in PRECISIONS.items()}[mode]


def svdp(A, k, which='LM', irl_mode=True, kmax=None, compute_u=True, compute_v=True, v0=None,
         full_output=False, tol=0, delta=None, eta=None, anorm=0, cgs=False, elr=True, min_relgap=0.002,
         shifts=None, maxiter=None, rng=None, precision="fp64"):
    """Singular triplets of A by Lanczos bidiagonalisation on the GPU.

    Argument semantics, defaults, validation and return values follow
    scipy.sparse.linalg._svdp._svdp (scipy/sparse/linalg/_svdp.py); the
    Fortran-level call follows double/dlansvd_irl.F:1-3 / dlansvd.F:1-3.
    precision: 'fp64' (default; the reference's method), 'mixed' (FP32
    Lanczos vectors, FP64 scalars, FP64 refinement to the requested tol) or
    'fp32' (the FP32 form alone, tol no finer than 16 * 2^-24: the form of
    the single-precision drivers slansvd_ / slansvd_irl_).
    Complex A (a complex CsrOperator, sparse or dense matrix, or a complex
    LinearOperator) runs the complex*16 drivers zlansvd_irl_ / zlansvd_
    (complex16/zlansvd_irl.F, zlansvd.F) in FP64, with scipy's complex start
    vector (uniform real and imaginary parts).
    Returns (u, sigma, vt, bnd) like scipy's _svdp."""
    from scipy.linalg import LinAlgError
    if rng is None:
        raise ValueError("`rng` must be a normalized numpy.random.Generator instance")
    which = which.upper()
    if which not in {'LM', 'SM'}:
        raise ValueError("`which` must be either 'LM' or 'SM'")
    if not irl_mode and which == 'SM':
        raise ValueError("`which`='SM' requires irl_mode=True")
    own_op = None
    if isinstance(A, CsrOperator):
        op = A
        cplx = op.dtype == np.complex128
    elif callable(getattr(A, "matvec", None)) and not hasattr(A, "tocsr"):
        op = None
        dt = getattr(A, "dtype", None)
        cplx = dt is not None and np.dtype(dt).kind == 'c'
    else:
        import scipy.sparse as sp
        op = own_op = CsrOperator(A)
        cplx = op.dtype == np.complex128
    if cplx and precision != "fp64":
        raise ValueError("complex matrices run in FP64 only (zlansvd_ / zlansvd_irl_)")
    m, n = op.shape if op is not None else A.shape
    if (k < 1) or (k > min(m, n)):
        raise ValueError("k must be positive and not greater than m or n")
    if kmax is None:
        kmax = 10 * k
    if maxiter is None:
        maxiter = 1000
    kmax = min(m + 1, n + 1, kmax)
    if kmax < k:
        raise ValueError("kmax must be greater than or equal to k, "
                         f"but kmax ({kmax}) < k ({k})")
    jobu = b'y' if compute_u else b'n'
    jobv = b'y' if compute_v else b'n'
    typ = np.complex128 if cplx else np.float64
    u = np.zeros((m, kmax + 1), order='F', dtype=typ)
    v = np.zeros((n, kmax), order='F', dtype=typ)
    sigma = np.zeros(k)
    bnd = np.zeros(k)
    if v0 is None:
        u[:, 0] = rng.uniform(size=m)
        if cplx:
            # scipy's start vector for complex input: uniform real and imaginary parts
            u[:, 0] += 1j * rng.uniform(size=m)
    else:
        try:
            u[:, 0] = v0
        except ValueError:
            raise ValueError(f"v0 must be of length {m}")
    if delta is None:
        delta = np.sqrt(np.finfo(np.float64).eps)
    if eta is None:
        eta = np.finfo(np.float64).eps ** 0.75
    if irl_mode:
        doption = np.array((delta, eta, anorm, min_relgap), dtype=np.float64)
        if shifts is None:
            shifts = kmax - k
        if k > min(kmax - shifts, m, n):
            raise ValueError('shifts must satisfy k <= min(kmax-shifts, m, n)!')
        elif shifts < 0:
            raise ValueError('shifts must be >= 0!')
    else:
        doption = np.array((delta, eta, anorm), dtype=np.float64)
    ioption = np.array((int(bool(cgs)), int(bool(elr))), dtype=np.int32)
    if op is not None:
        aprod, iparm = op.aprod, op.iparm
    else:
        aprod, iparm = (_host_zaprod(A) if cplx else _host_aprod(A)), None
    previous = get_precision()
    set_precision(precision)
    try:
        if cplx and irl_mode:
            kc, info = zlansvd_irl(_which_converter[which], jobu, jobv, m, n, kmax, shifts, k, maxiter, aprod,
                                   u, sigma, bnd, v, tol, doption, ioption, iparm=iparm)
        elif cplx:
            kc, info = zlansvd(jobu, jobv, m, n, k, kmax, aprod, u, sigma, bnd, v, tol, doption, ioption,
                               iparm=iparm)
        elif irl_mode:
            kc, info = lansvd_irl(_which_converter[which], jobu, jobv, m, n, kmax, shifts, k, maxiter, aprod,
                                  u, sigma, bnd, v, tol, doption, ioption, iparm=iparm)
        else:
            kc, info = lansvd(jobu, jobv, m, n, k, kmax, aprod, u, sigma, bnd, v, tol, doption, ioption,
                              iparm=iparm)
    finally:
        set_precision(previous)
        if own_op is not None:
            own_op.close()
    if info <= ERR_ARG:
        raise PropackError(f"GPU driver failed (INFO={info}): {last_error()}")
    if info > 0:
        raise LinAlgError(f"An invariant subspace of dimension {info} was found.")
    elif info < 0:
        raise LinAlgError(f"k={k} singular triplets did not converge within kmax={kmax} iterations")
    # scipy's _svdp returns the bounds whatever full_output says
    return u[:, :k], sigma, v[:, :k].conj().T, bnd
