"""Generate the golden fixtures of the complex*16 oracle.

scipy packages PROPACK's complex16 drivers (scipy.sparse.linalg._svdp._svdp
calls zlansvd / zlansvd_irl for complex input).  The non-restarted driver
is recorded as is (singular values, bounds and vectors).  The restarted
driver as shipped in scipy returns wrong singular values on these inputs
(relative errors of 0.4 to 0.8 against the dense SVD, for every kmax
tried), so the restarted cases are pinned to the dense SVD instead; their
scipy values are stored only to document that.  Inputs are stored with the
outputs, except the reference's example matrix mhd1280b, which comes from
scipy's own test data (propack_test_data.npz) wherever the tests run.
Run from the repository root:
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

# 3. the reference's complex example matrix mhd1280b (1280 x 1280, PROPACK's
# Examples/mhd1280b.cua, shipped in scipy's test data): the non-restarted
# driver at scipy's test configuration (k=200), and the restarted one at
# k=50, kmax=120, where it converges without a restart and, like any
# single-vector Lanczos run, misses copies of the repeated value 2
import scipy.sparse.linalg as sla  # noqa: E402
path = os.path.join(os.path.dirname(sla.__file__), "tests", "propack_test_data.npz")
with np.load(path, allow_pickle=True) as d:
    MHD = sp.csr_array(d["A_complex"].item())
u, s, vh, bnd = _svdp(MHD, 200, irl_mode=False, rng=np.random.default_rng(0), full_output=True)[:4]
out["mhd_lansvd_sigma"] = s
out["mhd_lansvd_bnd"] = bnd
out["mhd_irl50_sigma"] = _svdp(MHD, 50, irl_mode=True, kmax=120, tol=1e-10, rng=np.random.default_rng(0))[1]
out["mhd_dense_sigma"] = np.linalg.svd(MHD.toarray(), compute_uv=False)[:200]
print("mhd1280b", s[:3], "irl50 misses", np.sum(np.abs(out["mhd_irl50_sigma"] - out["mhd_dense_sigma"][:50]) > 1e-8))

np.savez_compressed(os.path.join(HERE, "golden_complex.npz"), **out)
print("wrote", os.path.join(HERE, "golden_complex.npz"))
