"""Batched solves: many independent sparse matrices in one persistent GPU
kernel (propack_batch_* in include/propack_gb300.h).

Every problem is solved by dlansvd_irl (double/dlansvd_irl.F) with full
reorthogonalisation, iterated classical Gram-Schmidt, FP64 vectors and the
matrix values in FP32; problems that the batched kernel hands back (an
invariant subspace, or Ritz values too close for its vector method) are
solved again by the single-problem driver with the same options and start
vector, so every returned problem is solved.
"""
import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import PropackError, last_error, load, svdp

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_i64p = C.POINTER(C.c_int64)
_fp = C.POINTER(C.c_float)


class BatchStats(C.Structure):
    _fields_ = [("nopx", C.c_int64), ("nreorth", C.c_int64), ("converged", C.c_int64), ("fallback", C.c_int64),
                ("device_ms", C.c_double), ("cycles", C.c_int64), ("grid", C.c_int64),
                ("kernel_launches", C.c_int64), ("tune_ms", C.c_double)]

NCLASS = 4  # PROPACK_BATCH_CLASSES: size classes of the autotuner


def _lib():
    L = load()
    if not getattr(L, "_batch_bound", False):
        L.propack_batch_create.argtypes = [C.c_int, _ip, _ip, _ip, _i64p, _ip, _fp, _i64p]
        L.propack_batch_destroy.argtypes = [C.c_int64]
        L.propack_batch_solve.argtypes = [C.c_int64, C.c_int, C.c_int, C.c_int, C.c_double, _dp, _dp, _dp, _ip,
                                          _dp, _dp]
        L.propack_batch_get_stats.argtypes = [C.POINTER(BatchStats)]
        L.propack_batch_get_tuning.argtypes = [C.c_int64, _ip, _ip, _fp, _fp]
        L.propack_batch_set_tuning.argtypes = [C.c_int64, _ip, _ip]
        L.propack_batch_set_arith.argtypes = [C.c_int64, C.c_int]
        L._batch_bound = True
    return L


class Batch:
    """A set of CSR matrices resident on the GPU (values stored as FP32)."""

    def __init__(self, mats):
        self._L = _lib()
        self.mats = [sp.csr_array(A) for A in mats]
        for A in self.mats:
            A.sort_indices()
        self.m = np.array([A.shape[0] for A in self.mats], dtype=np.int32)
        self.n = np.array([A.shape[1] for A in self.mats], dtype=np.int32)
        nnz = np.array([A.nnz for A in self.mats], dtype=np.int64)
        self.nnz_off = np.zeros(len(self.mats) + 1, dtype=np.int64)
        np.cumsum(nnz, out=self.nnz_off[1:])
        rowptr = np.concatenate([A.indptr.astype(np.int32) for A in self.mats])
        colidx = np.concatenate([A.indices.astype(np.int32) for A in self.mats])
        val = np.concatenate([A.data.astype(np.float32) for A in self.mats])
        h = C.c_int64(0)
        rc = self._L.propack_batch_create(len(self.mats), self.m.ctypes.data_as(_ip), self.n.ctypes.data_as(_ip),
                                          rowptr.ctypes.data_as(_ip), self.nnz_off.ctypes.data_as(_i64p),
                                          colidx.ctypes.data_as(_ip), val.ctypes.data_as(_fp), C.byref(h))
        if rc != 0:
            raise PropackError(f"propack_batch_create failed ({rc}): {last_error()}")
        self.handle = h.value

    def tuning(self):
        """The autotuner's table: per size class (quarters of the batch by
        decreasing size) the SpMV row split g, the projection tile dc and the
        probe's ms with them and with (1, 1); state 0 untuned, 1 timed, 2 set."""
        g = np.zeros(NCLASS, dtype=np.int32)
        dc = np.zeros(NCLASS, dtype=np.int32)
        mt = np.zeros(NCLASS, dtype=np.float32)
        md = np.zeros(NCLASS, dtype=np.float32)
        st = self._L.propack_batch_get_tuning(self.handle, g.ctypes.data_as(_ip), dc.ctypes.data_as(_ip),
                                              mt.ctypes.data_as(_fp), md.ctypes.data_as(_fp))
        if st < 0:
            raise PropackError(f"propack_batch_get_tuning failed ({st}): {last_error()}")
        return {"state": st, "g": g.tolist(), "dc": dc.tolist(), "probe_ms": mt.tolist(),
                "probe_ms_default": md.tolist()}

    def set_tuning(self, g=None, dc=None):
        """Pin the table (lists of NCLASS values), or with no arguments ask
        for a new timing at the next solve."""
        if g is None or dc is None:
            rc = self._L.propack_batch_set_tuning(self.handle, None, None)
        else:
            ga = np.ascontiguousarray(g, dtype=np.int32)
            da = np.ascontiguousarray(dc, dtype=np.int32)
            rc = self._L.propack_batch_set_tuning(self.handle, ga.ctypes.data_as(_ip), da.ctypes.data_as(_ip))
        if rc != 0:
            raise PropackError(f"propack_batch_set_tuning failed ({rc}): {last_error()}")

    def set_arith(self, arith):
        """Arithmetic of the products and Gram-Schmidt passes: "fp64" (the
        default) or "planes" (FP32 (hi, lo) planes of the bases;
        propack_batch_set_arith)."""
        rc = self._L.propack_batch_set_arith(self.handle, {"fp64": 0, "planes": 2}[arith])
        if rc != 0:
            raise PropackError(f"propack_batch_set_arith failed ({rc})")

    def close(self):
        if self.handle:
            self._L.propack_batch_destroy(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, k, kmax=40, tol=1e-8, maxiter=100, u0=None, rng=None, vectors=True):
        """Top-k triplets of every matrix.  Returns (sigma (nprob x k),
        bnd (nprob x k), info (nprob), U list, V list) -- info 0 converged,
        -1 not converged within maxiter; problems the kernel handed back are
        re-solved by the single-problem driver (info from that solve)."""
        np_ = len(self.mats)
        if u0 is None:
            rng = np.random.default_rng(0) if rng is None else rng
            u0 = [rng.uniform(size=int(m)) for m in self.m]
        u0c = np.ascontiguousarray(np.concatenate(u0), dtype=np.float64)
        sig = np.zeros((np_, k))
        bnd = np.zeros((np_, k))
        info = np.zeros(np_, dtype=np.int32)
        Ub = np.zeros(int(self.m.sum()) * k) if vectors else None
        Vb = np.zeros(int(self.n.sum()) * k) if vectors else None
        rc = self._L.propack_batch_solve(self.handle, kmax, k, maxiter, tol, u0c.ctypes.data_as(_dp),
                                         sig.ctypes.data_as(_dp), bnd.ctypes.data_as(_dp),
                                         info.ctypes.data_as(_ip), Ub.ctypes.data_as(_dp) if vectors else None,
                                         Vb.ctypes.data_as(_dp) if vectors else None)
        if rc != 0:
            raise PropackError(f"propack_batch_solve failed ({rc}): {last_error()}")
        self.stats = stats()
        U, V = [], []
        mo = no = 0
        for p in range(np_):
            m, n = int(self.m[p]), int(self.n[p])
            if vectors:
                U.append(Ub[mo * k:(mo + m) * k].reshape(k, m).T.copy())
                V.append(Vb[no * k:(no + n) * k].reshape(k, n).T.copy())
            mo += m
            no += n
            if info[p] == 1:
                u, s, vt, b = svdp(self.mats[p], k, kmax=kmax, tol=tol, maxiter=maxiter, v0=u0[p], cgs=True,
                                   delta=0.0, eta=0.0)
                sig[p], bnd[p], info[p] = s, b, 0
                if vectors:
                    U[p], V[p] = u, vt.T
        return sig, bnd, info, U, V


def stats():
    s = BatchStats()
    _lib().propack_batch_get_stats(C.byref(s))
    return {k: getattr(s, k) for k, _ in BatchStats._fields_}


def random_batch(nprob, m_range=(500, 20000), n_range=(200, 8000), density=0.01, seed=3):
    """Independent CSR matrices with uniform sizes, Bernoulli(density) rows
    of uniform columns and N(0,1) values stored as FP32."""
    rng = np.random.default_rng(seed)
    mats = []
    for _ in range(nprob):
        m = int(rng.integers(m_range[0], m_range[1] + 1))
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        cnt = rng.binomial(n, density, size=m).astype(np.int64)
        indptr = np.zeros(m + 1, dtype=np.int64)
        np.cumsum(cnt, out=indptr[1:])
        nnz = int(indptr[-1])
        idx = rng.integers(0, n, size=nnz, dtype=np.int32)
        val = rng.standard_normal(nnz).astype(np.float32).astype(np.float64)
        A = sp.csr_array((val, idx, indptr), shape=(m, n))
        A.sum_duplicates()
        A.data = A.data.astype(np.float32).astype(np.float64)  # merged duplicates back to FP32 values
        mats.append(A)
    return mats


__all__ = ["Batch", "stats", "random_batch"]
