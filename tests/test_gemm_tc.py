"""The FP64 restart/Ritz product on the tensor cores (error-free digit
split, dlansvd_irl.F:371-398, dritzvec.F:130-198): the tcgen05 kernels
(barrier-staged and warp-specialised) and the mma.sync kernel must give the
same bits, and all must match an FP64
product to the split's error bound (operands kept to 2^-49 of their row and
column maxima, digit products below 2^-56 dropped; the level sums
themselves are exact)."""
import ctypes as C

import numpy as np
import pytest

import propack_gb300 as pg

pytestmark = pytest.mark.gpu

_dp = C.POINTER(C.c_double)


def _call(impl, A_t, lda, B_t, ldb, tb, C_t, ldc, mr, nc, kk):
    L = pg.load()
    L.propack_gemm_f64_tc.restype = C.c_int
    L.propack_gemm_f64_tc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                      C.c_int, C.c_void_p, C.c_int]
    rc = L.propack_gemm_f64_tc(impl, mr, nc, kk, A_t.data_ptr(), lda, B_t.data_ptr(), ldb, tb, C_t.data_ptr(), ldc)
    assert rc == 0, pg.last_error()


@pytest.mark.parametrize("mr,kk,nc,tb", [(4133, 151, 50, 0), (4096, 151, 51, 1), (8200, 33, 65, 0),
                                         (5000, 256, 130, 1), (4500, 1, 7, 0), (4097, 40, 64, 1)])
def test_tcgen05_matches_mma_sync_and_fp64(mr, kk, nc, tb):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(mr + kk + nc)
    lda, ldb, ldc = mr + 3, (nc if tb else kk) + 1, mr + 1
    A = rng.standard_normal((mr, kk)) * 10.0 ** rng.uniform(-3, 3, (mr, 1))
    A[rng.random(mr) < 0.01] = 0.0
    A[5, :] = 0.0
    A[7, 0] = 1e-300  # a tiny entry beside normal ones: its digits drop out
    Bop = rng.standard_normal((kk, nc)) * 10.0 ** rng.uniform(-2, 2, (1, nc))
    Amem = np.zeros((kk, lda))
    Amem[:, :mr] = A.T
    if tb:
        Bmem = np.zeros((kk, ldb))
        Bmem[:, :nc] = Bop
    else:
        Bmem = np.zeros((nc, ldb))
        Bmem[:, :kk] = Bop.T
    dev = torch.device("cuda:0")
    A_t = torch.from_numpy(Amem).to(dev)
    B_t = torch.from_numpy(Bmem).to(dev)
    outs = []
    for impl in (0, 1, 2):
        C_t = torch.full((nc, ldc), np.nan, dtype=torch.float64, device=dev)
        _call(impl, A_t, lda, B_t, ldb, tb, C_t, ldc, mr, nc, kk)
        Cm = C_t.cpu().numpy()
        assert np.all(np.isnan(Cm[:, mr:]))  # rows past mr untouched
        outs.append(Cm[:, :mr].T)
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[1], outs[2])
    # the split keeps every operand to 2^-49 of its row (column) maximum and
    # drops the digit products below 2^-56: |error| <= K 2^-45 max|A(i,:)| max|B(:,j)|
    ref = A @ Bop
    bound = kk * 2.0 ** -45 * np.outer(np.abs(A).max(axis=1), np.abs(Bop).max(axis=0)) + 1e-300
    assert np.all(np.abs(outs[1] - ref) <= bound)


def test_aligned_signs_take_the_wide_path():
    # every product of a row and a column equal: the top level reaches
    # K * 64 * 64 > 2^19 and the levels are combined in two parts
    torch = pytest.importorskip("torch")
    mr, kk, nc = 4100, 151, 3
    dev = torch.device("cuda:0")
    A_t = torch.ones((kk, mr), dtype=torch.float64, device=dev)
    B_t = torch.ones((nc, kk), dtype=torch.float64, device=dev)
    for impl in (0, 1, 2):
        C_t = torch.zeros((nc, mr), dtype=torch.float64, device=dev)
        _call(impl, A_t, mr, B_t, kk, 0, C_t, mr, mr, nc, kk)
        assert torch.all(C_t == float(kk))


def test_warp_specialised_kernel_in_the_solve():
    """The drivers' restart products on either tcgen05 kernel give the same
    bits (propack_set_gemm_impl)."""
    pytest.importorskip("torch")
    import scipy.sparse as sp
    rng = np.random.default_rng(4)
    A = sp.random_array((6000, 1500), density=0.004, format="csr", random_state=rng)
    out = []
    try:
        for impl in (1, 2):
            assert pg.load().propack_set_gemm_impl(impl) == 0
            u, s, vt, bnd = pg.svdp(A, 6, irl_mode=True, kmax=24, tol=1e-10, rng=np.random.default_rng(0))
            assert pg.get_stats()["nrestart"] > 0
            out.append((u, s, vt))
    finally:
        pg.load().propack_set_gemm_impl(2)
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
