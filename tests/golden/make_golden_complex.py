"""Generate the golden fixtures of the complex*16 oracle.

scipy packages PROPACK's complex16 drivers (scipy.sparse.linalg._svdp._svdp
calls zlansvd / zlansvd_irl for complex input).  The non-restarted driver
is recorded as is (singular values, bounds and vectors).  The restarted
driver as shipped in scipy returns wrong singular values on these inputs
(relative errors of 0.4 to 0.8 against the dense SVD, for every kmax
tried), so the restarted cases are pinned to the dense SVD instead; their
scipy values are stored only to document that.  Inputs are stored with the
outputs.  Run from the repository root:
    python tests/golden/make_golden_complex.py
"""
import os

import numpy as np
import scipy
import scipy.sparse as sp
from scipy.sparse.linalg._svdp import _svdp

HERE = os.path.dirname(os.path.abspath(__file__))
out = {"scipy_version": np.array(scipy.__version__)}


def put_csr(prefix, A):
    A = sp.csr_array(A)
    out[prefix + "_shape"] = np.array(A.shape)
    out[prefix + "_indptr"] = A.indptr.astype(np.int64)
    out[prefix + "_indices"] = A.indices.astype(np.int32)
    out[prefix + "_data"] = A.data.astype(np.complex128)


def run(name, A, k, **kw):
    u, s, vh, bnd = _svdp(A, k, rng=np.random.default_rng(0), full_output=True, **kw)[:4]
    out[name + "_sigma"] = s
    out[name + "_bnd"] = bnd
    out[name + "_u"] = u
    out[name + "_vh"] = vh
    print(name, s[:5])


def complex_matrix(m, n, density, seed):
    rng = np.random.default_rng(seed)
    re = sp.random(m, n, density=density, random_state=rng, format="csr")
    mask = re.copy()
    mask.data = rng.standard_normal(mask.nnz) + 1j * rng.standard_normal(mask.nnz)
    return sp.csr_array(mask)


# 1. a small complex matrix: non-restarted driver with MGS and with CGS
Z1 = complex_matrix(300, 200, 0.05, 1)
put_csr("z1", Z1)
run("z1_lansvd", Z1, 5, irl_mode=False, kmax=80, tol=1e-12)
run("z1_lansvd_cgs", Z1, 5, irl_mode=False, kmax=80, tol=1e-12, cgs=True)
out["z1_dense_sigma"] = np.linalg.svd(Z1.toarray(), compute_uv=False)[:20]
s_irl = _svdp(Z1, 5, irl_mode=True, kmax=30, tol=1e-12, rng=np.random.default_rng(0))[1]
out["z1_irl_scipy_sigma"] = s_irl
print("z1 irl (scipy)", s_irl, "dense", out["z1_dense_sigma"][:5])

# 2. a wide complex matrix (n > m: the initial anorm estimate goes through A)
Z2 = complex_matrix(150, 400, 0.04, 2)
put_csr("z2", Z2)
run("z2_lansvd", Z2, 6, irl_mode=False, kmax=120, tol=1e-12)
out["z2_dense_sigma"] = np.linalg.svd(Z2.toarray(), compute_uv=False)[:20]

np.savez_compressed(os.path.join(HERE, "golden_complex.npz"), **out)
print("wrote", os.path.join(HERE, "golden_complex.npz"))
