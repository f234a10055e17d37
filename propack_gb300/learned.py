"""Learned start vector: a row-wise MLP that proposes U(:,1) for the
Lanczos bidiagonalisation in place of dgetu0's random start
(double/dgetu0.F:11-89).

The network, its features and its loss are described in
include/propack_gb300.h (propack_mlp_*); forward and backward passes and the
Adam update run on the GPU in the library's own kernels.  The random start
stays both the fallback and the arbiter: a solve from the learned start whose
own Ritz error bounds (``bnd <= tol * sigma``, the convergence test of
dlansvd_irl.F:281) do not certify all k triplets is repeated from the random
start.
"""
import ctypes as C

import numpy as np

from scipy.linalg import LinAlgError

from . import CsrOperator, PropackError, get_stats, last_error, load, svdp

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


def _lib():
    L = load()
    if not getattr(L, "_mlp_bound", False):
        L.propack_mlp_create.argtypes = [C.c_uint64, C.POINTER(C.c_int64)]
        L.propack_mlp_destroy.argtypes = [C.c_int64]
        L.propack_mlp_nparams.restype = C.c_int
        L.propack_mlp_params.argtypes = [C.c_int64, _fp, _fp]
        L.propack_mlp_features.argtypes = [C.c_int64, C.c_int64, C.c_uint64, _fp]
        L.propack_mlp_start.argtypes = [C.c_int64, C.c_int64, C.c_uint64, _dp]
        L.propack_mlp_grad.argtypes = [C.c_int64, C.c_int64, C.c_uint64, _dp, C.c_int, C.c_int, _fp, _dp]
        L.propack_mlp_set_impl.argtypes = [C.c_int]
        L.propack_mlp_train_step.argtypes = [C.c_int64, C.c_int64, C.c_uint64, _dp, C.c_int, C.c_int, C.c_double,
                                             _dp]
        L._mlp_bound = True
    return L


def set_layer_impl(impl):
    """The 256 x 256 layer's kernel (process-wide): "tcgen05" (default) or
    "mma_sync" (the reference implementation)."""
    _check(_lib().propack_mlp_set_impl({"mma_sync": 0, "tcgen05": 1}[impl]), "propack_mlp_set_impl")


def _check(rc, what):
    if rc != 0:
        raise PropackError(f"{what} failed ({rc}): {last_error()}")


class StartModel:
    """The learned start vector model (one per device)."""

    def __init__(self, seed=0, sketch_seed=12345):
        self._L = _lib()
        h = C.c_int64(0)
        _check(self._L.propack_mlp_create(seed, C.byref(h)), "propack_mlp_create")
        self.handle = h.value
        self.sketch_seed = sketch_seed
        self.nparams = self._L.propack_mlp_nparams()

    def close(self):
        if self.handle:
            self._L.propack_mlp_destroy(self.handle)
            self.handle = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        out = np.zeros(self.nparams, dtype=np.float32)
        _check(self._L.propack_mlp_params(self.handle, out.ctypes.data_as(_fp), None), "propack_mlp_params")
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        _check(self._L.propack_mlp_params(self.handle, None, p.ctypes.data_as(_fp)), "propack_mlp_params")

    def features(self, op):
        F = np.zeros((op.shape[0], 18), dtype=np.float32)
        _check(self._L.propack_mlp_features(self.handle, op.handle, self.sketch_seed, F.ctypes.data_as(_fp)),
               "propack_mlp_features")
        return F

    def start(self, op):
        """Proposed start vector for the operator (unit norm)."""
        u0 = np.zeros(op.shape[0])
        _check(self._L.propack_mlp_start(self.handle, op.handle, self.sketch_seed, u0.ctypes.data_as(_dp)),
               "propack_mlp_start")
        nrm = np.linalg.norm(u0)
        return u0 / nrm if nrm > 0 else u0

    def _U(self, U):
        return np.asfortranarray(U, dtype=np.float64)

    def grad(self, op, U):
        """(loss, flat gradient) for (op, U) without an update."""
        U = self._U(U)
        g = np.zeros(self.nparams, dtype=np.float32)
        loss = C.c_double(0.0)
        _check(self._L.propack_mlp_grad(self.handle, op.handle, self.sketch_seed, U.ctypes.data_as(_dp), U.shape[0],
                                        U.shape[1], g.ctypes.data_as(_fp), C.byref(loss)), "propack_mlp_grad")
        return loss.value, g

    def train_step(self, op, U, lr=1e-3):
        U = self._U(U)
        loss = C.c_double(0.0)
        _check(self._L.propack_mlp_train_step(self.handle, op.handle, self.sketch_seed, U.ctypes.data_as(_dp),
                                              U.shape[0], U.shape[1], lr, C.byref(loss)), "propack_mlp_train_step")
        return loss.value


def solve(op, k, model=None, tol=1e-8, rng=None, **kw):
    """svdp(op, k) from the model's start vector, judged by the method's own
    Ritz error bounds and repeated from the random start when they fail.
    Returns (u, sigma, vt, bnd, info) with info = {"start": "learned" |
    "random" | "random-fallback", "nopx": matvecs of all solves}."""
    rng = np.random.default_rng(0) if rng is None else rng
    nopx = 0
    if model is not None:
        u0 = model.start(op)
        if np.all(np.isfinite(u0)) and np.linalg.norm(u0) > 0:
            try:
                u, s, vt, bnd = svdp(op, k, tol=tol, v0=u0, rng=rng, **kw)
                nopx += get_stats()["nopx"]
                if np.all(bnd <= tol * s):
                    return u, s, vt, bnd, {"start": "learned", "nopx": nopx}
            except LinAlgError:
                nopx += get_stats()["nopx"]
        u, s, vt, bnd = svdp(op, k, tol=tol, rng=rng, **kw)
        nopx += get_stats()["nopx"]
        return u, s, vt, bnd, {"start": "random-fallback", "nopx": nopx}
    u, s, vt, bnd = svdp(op, k, tol=tol, rng=rng, **kw)
    return u, s, vt, bnd, {"start": "random", "nopx": get_stats()["nopx"]}


__all__ = ["StartModel", "solve", "CsrOperator"]
