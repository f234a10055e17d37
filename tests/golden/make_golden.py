"""Generate the golden fixtures of the parity tests.

The reference algorithm is run through scipy's packaging of PROPACK
(scipy.sparse.linalg._svdp._svdp, which calls PROPACK's dlansvd /
dlansvd_irl).  Inputs are stored with the outputs so that the fixtures do
not depend on the numpy random streams of the machine that replays them.
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np
import scipy
import scipy.sparse as sp
from scipy.sparse.linalg._svdp import _svdp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from propack_gb300 import workloads  # noqa: E402

out = {"scipy_version": np.array(scipy.__version__)}


def put_csr(prefix, A):
    A = sp.csr_array(A)
    out[prefix + "_shape"] = np.array(A.shape)
    out[prefix + "_indptr"] = A.indptr.astype(np.int64)
    out[prefix + "_indices"] = A.indices.astype(np.int32)
    out[prefix + "_data"] = A.data.astype(np.float64)


def run(name, A, k, vectors=True, **kw):
    u, s, vt, bnd = _svdp(A, k, rng=np.random.default_rng(0), **kw)
    out[name + "_sigma"] = s
    out[name + "_bnd"] = bnd
    if vectors:
        out[name + "_u"] = u
        out[name + "_vt"] = vt
    # the start vector scipy used (u[:,0] = rng.uniform(size=m))
    out[name + "_u0"] = np.random.default_rng(0).uniform(size=A.shape[0])
    print(name, s[:5])


# 1. the CPU-runnable plain DLANSVD configuration (2000 x 1000, k=10)
A0 = workloads.plain_lansvd(0)
put_csr("plain", A0)
run("plain_lansvd", A0, 10, irl_mode=False, kmax=200, tol=1e-12)
run("plain_irl", A0, 10, irl_mode=True, kmax=30, tol=1e-12)
out["plain_dense_sigma"] = np.linalg.svd(A0.toarray(), compute_uv=False)[:20]

# 2. scipy's own small cases (test_propack.py check_svdp matrix: n=10, m=20)
rng2 = np.random.default_rng(0)
M = -5 + 10 * rng2.uniform(size=[10, 20])
M[M > 10 * 0.8 - 5] = 0
put_csr("small", M)
run("small_irl_lm", M, 3, irl_mode=True, which='LM', tol=1e-8)
run("small_irl_sm", M, 3, irl_mode=True, which='SM', tol=1e-8)
run("small_lansvd", M, 3, irl_mode=False, tol=1e-8)

# 3. a small instance of the low-rank IRL configuration (restarts, ELR, partial reorth)
S, L, R, w = workloads.lowrank_irl(seed=11, m=6000, n=1500, nnz_row=20, rank=8, udens=0.05, vdens=0.1)
Ad = workloads.dense_of(S, L, R, w)
put_csr("lr_S", S)
put_csr("lr_L", L)
put_csr("lr_R", R)
out["lr_w"] = w
run("lowrank_irl", sp.csr_array(Ad), 10, irl_mode=True, kmax=30, tol=1e-10)
out["lowrank_dense_sigma"] = np.linalg.svd(Ad, compute_uv=False)[:20]

# 4. illc1850 (the reference's own example matrix, shipped with scipy's tests):
#    only the outputs are stored; the test reads the matrix from scipy if present.
path = os.path.join(os.path.dirname(scipy.sparse.linalg.__file__), "tests", "propack_test_data.npz")
if os.path.exists(path):
    with np.load(path, allow_pickle=True) as data:
        Ai = sp.csr_array(data["A_real"].item())
    u, s, vt, bnd = _svdp(Ai, 200, irl_mode=False, rng=np.random.default_rng(0))
    out["illc_sigma"] = s
    out["illc_dense_sigma"] = np.linalg.svd(Ai.toarray(), compute_uv=False)[:200]
    print("illc1850", s[:3])

np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
print("wrote", os.path.join(HERE, "golden.npz"))
