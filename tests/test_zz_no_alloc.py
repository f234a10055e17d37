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


def test_noalloc_takes_no_device_memory_after_warm_up():
    # the property the entry point exists for: once a first call has loaded
    # the kernels and looked up the scratch address, further calls leave the
    # device's free memory and torch's allocator untouched
    torch = pytest.importorskip("torch")
    lib = pg.load()
    S, L, R, w = workloads.lowrank_irl(seed=22, m=20000, n=6000, nnz_row=10, rank=8, udens=0.05, vdens=0.1)
    op = pg.CsrOperator(S, L, R, w)
    m, n = op.shape
    xd = torch.ones(n, dtype=torch.float64, device="cuda")
    yd = torch.zeros(m, dtype=torch.float64, device="cuda")
    assert _noalloc(lib, op.handle, 0, xd.data_ptr(), yd.data_ptr()) == 0, pg.last_error()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    alloc0 = torch.cuda.memory_stats().get("allocated_bytes.all.current", 0)
    for _ in range(3):
        assert _noalloc(lib, op.handle, 0, xd.data_ptr(), yd.data_ptr()) == 0, pg.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_stats().get("allocated_bytes.all.current", 0) == alloc0
    np.testing.assert_allclose(yd.cpu().numpy(), op.matvec(np.ones(n)), rtol=1e-12, atol=1e-12)
    op.close()


def test_noalloc_refuses_host_pointers():
    # a host buffer passed by mistake is refused (cudaPointerGetAttributes,
    # before any launch) instead of faulting in a kernel
    torch = pytest.importorskip("torch")
    lib = pg.load()
    S, L, R, w = workloads.lowrank_irl(seed=23, m=3000, n=1000, nnz_row=6, rank=4, udens=0.05, vdens=0.1)
    op = pg.CsrOperator(S, L, R, w)
    m, n = op.shape
    xh = np.ones(n)
    yd = torch.zeros(m, dtype=torch.float64, device="cuda")
    rc = _noalloc(lib, op.handle, 0, xh.ctypes.data, yd.data_ptr())
    assert rc == pg.ERR_ARG and "device" in pg.last_error()
    xd = torch.ones(n, dtype=torch.float64, device="cuda")
    yh = np.zeros(m)
    assert _noalloc(lib, op.handle, 0, xd.data_ptr(), yh.ctypes.data) == pg.ERR_ARG
    op.close()


@pytest.mark.parametrize("form", ["native", "block"])
def test_noalloc_complex_operator(form):
    # a complex operator (native complex CSR, or the real 2x2-block form)
    # takes interleaved (re, im) doubles and applies A (trans 0) or A^H
    # (trans 1), twice in a row; the native form refuses vectors that are
    # not 16-byte aligned before any launch
    torch = pytest.importorskip("torch")
    import scipy.sparse as sp
    lib = pg.load()
    rng = np.random.default_rng(7)
    m, n, k = 700, 500, 6
    rows = np.repeat(np.arange(m), k)
    A = sp.csr_array((rng.standard_normal(m * k) + 1j * rng.standard_normal(m * k),
                      (rows, rng.integers(0, n, m * k))), shape=(m, n))
    pg.set_complex_form(form)
    try:
        op = pg.CsrOperator(A)
    finally:
        pg.set_complex_form("native")
    if form == "native":
        buf = torch.zeros(2 * max(m, n) + 2, dtype=torch.float64, device="cuda")
        assert _noalloc(lib, op.handle, 0, buf.data_ptr() + 8, buf.data_ptr()) == pg.ERR_ARG
        assert "aligned" in pg.last_error()
    for call in range(2):
        for trans in (0, 1):
            x = rng.standard_normal(m if trans else n) + 1j * rng.standard_normal(m if trans else n)
            ref = A.conj().T @ x if trans else A @ x
            xd = torch.tensor(x.view(np.float64), dtype=torch.float64, device="cuda")
            yd = torch.full((2 * (n if trans else m),), np.nan, dtype=torch.float64, device="cuda")
            assert _noalloc(lib, op.handle, trans, xd.data_ptr(), yd.data_ptr()) == 0, pg.last_error()
            torch.cuda.synchronize()
            got = yd.cpu().numpy().view(np.complex128)
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
