"""The allocation-free operator application (propack_csr_apply_noalloc).

It serves callers that may not allocate device memory while they run; its
scratch is a fixed array in device memory shared by all calls.  This file
is named so that pytest collects it last.  The test calls the entry point
through the C ABI on device vectors and compares the result with the
allocating entry point propack_gpu_csr_aprod_ on the same operator, for
two calls in a row (the shared scratch must not leak state from one call
into the next)."""
import ctypes as C

import numpy as np
import pytest

import propack_gb300 as pg
from propack_gb300 import workloads

pytestmark = pytest.mark.gpu


def _noalloc(lib, handle, trans, x_dev, y_dev):
    lib.propack_csr_apply_noalloc.restype = C.c_int
    lib.propack_csr_apply_noalloc.argtypes = [C.c_int64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    return lib.propack_csr_apply_noalloc(handle, trans, x_dev, y_dev, None)


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    lib = pg.load()
    S, L, R, w = workloads.lowrank_irl(seed=21, m=40000, n=9000, nnz_row=12, rank=16, udens=0.05, vdens=0.1)
    op = pg.CsrOperator(S, L, R, w)
    m, n = op.shape
    rng = np.random.default_rng(5)
    for call in range(2):
        for trans in (0, 1):
            x = rng.standard_normal(m if trans else n)
            ref = op.rmatvec(x) if trans else op.matvec(x)
            xd = torch.tensor(x, dtype=torch.float64, device="cuda")
            yd = torch.full((n if trans else m,), np.nan, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            rc = _noalloc(lib, op.handle, trans, xd.data_ptr(), yd.data_ptr())
            torch.cuda.synchronize()
            assert rc == 0, pg.last_error()
            got = yd.cpu().numpy()
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max(),
                                       err_msg=f"call {call}, trans {trans}")
    op.close()


def test_noalloc_rejects_scratch_beyond_the_limit():
    torch = pytest.importorskip("torch")
    import scipy.sparse as sp
    lib = pg.load()
    m, n, r = 300, 200, 40000   # r * (1 + segments) + 1 > 65536 doubles
    rng = np.random.default_rng(1)
    S = sp.csr_array((rng.standard_normal(m * 5), (np.repeat(np.arange(m), 5), rng.integers(0, n, m * 5))),
                     shape=(m, n))
    L = sp.csr_array((np.ones(r), (np.arange(r) % m, np.arange(r))), shape=(m, r))
    R = sp.csr_array((np.ones(r), (np.arange(r) % n, np.arange(r))), shape=(n, r))
    op = pg.CsrOperator(S, L, R, np.ones(r))
    xd = torch.zeros(n, dtype=torch.float64, device="cuda")
    yd = torch.zeros(m, dtype=torch.float64, device="cuda")
    rc = _noalloc(lib, op.handle, 0, xd.data_ptr(), yd.data_ptr())
    assert rc == pg.ERR_ARG
    assert "scratch" in pg.last_error()
    op.close()
