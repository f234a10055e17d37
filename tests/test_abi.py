"""The C-ABI library builds for sm_103a, loads, and exports every symbol that
include/propack_gb300.h declares (no compute calls: no GPU needed)."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "propack_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set()
    for m in re.finditer(r"\b(?:void|int|const char \*)\s*\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
        names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_reference_entry_points():
    names = declared_symbols()
    for n in ("dlansvd_", "dlansvd_irl_", "clearstat_", "printstat_", "propack_gpu_csr_aprod_",
              "propack_csr_create", "propack_csr_destroy", "slansvd_", "slansvd_irl_", "zlansvd_",
              "zlansvd_irl_", "propack_zcsr_create", "propack_gpu_csr_zaprod_"):
        assert n in names


def test_library_builds_and_exports_all_symbols():
    from propack_gb300 import _build
    lib = _build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [n for n in declared_symbols() if n not in exported]
    assert not missing, missing


def test_library_loads():
    import propack_gb300 as pg
    L = pg.load()
    for n in declared_symbols():
        assert hasattr(L, n)


def test_kernels_compiled_for_sm103a_only():
    # the build recipe compiles every translation unit and links for sm_103a
    # alone (the loaded kernels' binary version is checked on the GPU in
    # test_gpu_parity.py::test_loaded_kernels_are_sm103)
    from propack_gb300 import _build
    assert _build.GENCODE == ["-gencode", "arch=compute_103a,code=sm_103a"]


@pytest.mark.parametrize("driver", ["dlansvd_irl_", "dlansvd_", "zlansvd_irl_", "zlansvd_", "slansvd_irl_",
                                    "slansvd_"])
def test_short_workspace_is_refused_before_any_device_work(driver):
    """LWORK / LIWORK / LZWRK below what the reference's drivers write
    (double/dlansvd_irl.F:177-188, double/dlansvd.F:151-160) give INFO =
    PROPACK_ERR_ARG and a message naming the argument; the check runs before
    any CUDA call, so no GPU is needed."""
    import ctypes as C
    import propack_gb300 as pg
    L = pg.load()
    m, n, kmax, k = 300, 200, 20, 5
    irl = driver.endswith("_irl_")
    cplx = driver.startswith("z")
    single = driver.startswith("s")
    lw, liw, lzw = pg.work_sizes(m, n, kmax, irl=irl, cplx=cplx)
    ci = lambda v: C.byref(C.c_int(v))
    vp = lambda a: C.c_void_p(a.ctypes.data)
    ft = np.float32 if single else np.float64
    ct = np.complex128 if cplx else ft
    U = np.zeros((m, kmax + 1), dtype=ct, order="F")
    V = np.zeros((n, kmax), dtype=ct, order="F")
    sig, bnd = np.zeros(k, dtype=ft), np.zeros(k, dtype=ft)
    opt = np.zeros(4, dtype=ft)
    iop = np.array([0, 1], dtype=np.int32)
    iparm = np.zeros(2, dtype=np.int32)
    parm = np.zeros(2, dtype=ct)
    tol = C.byref(C.c_float(1e-5) if single else C.c_double(1e-8))
    aprod = C.c_void_p(C.cast(L.propack_gpu_csr_zaprod_ if cplx else (L.propack_gpu_csr_saprod_ if single
                                                                          else L.propack_gpu_csr_aprod_),
                              C.c_void_p).value)
    for bad in ("lwork", "liwork") + (("lzwrk",) if cplx else ()):
        sizes = {"lwork": lw, "liwork": liw, "lzwrk": lzw}
        sizes[bad] = 3
        work = np.empty(sizes["lwork"], dtype=ft)
        iwork = np.empty(sizes["liwork"], dtype=np.int32)
        zwork = np.empty(max(sizes["lzwrk"], 1), dtype=np.complex128)
        info, kk = C.c_int(0), C.c_int(k)
        head = [C.c_char_p(b"y"), C.c_char_p(b"y"), ci(m), ci(n)]
        if irl:
            head = [C.c_char_p(b"L")] + head + [ci(kmax), ci(kmax - k), C.byref(kk), ci(10)]
        else:
            head = head + [C.byref(kk), ci(kmax)]
        mid = [aprod, vp(U), ci(m), vp(sig), vp(bnd), vp(V), ci(n), tol, vp(work), ci(sizes["lwork"])]
        if cplx:
            mid += [vp(zwork), ci(sizes["lzwrk"])]
        tail = [vp(iwork), ci(sizes["liwork"]), vp(opt), vp(iop), C.byref(info), vp(parm), vp(iparm)]
        lens = [C.c_size_t(1)] * (3 if irl else 2)
        getattr(L, driver)(*(head + mid + tail + lens))
        assert info.value == pg.ERR_ARG, (driver, bad, info.value)
        assert bad.upper() in pg.last_error(), pg.last_error()


def test_svdp_argument_validation_matches_scipy():
    import numpy as np
    import propack_gb300 as pg
    A = np.ones((5, 4))
    with pytest.raises(ValueError):
        pg.svdp(A, 3, rng=None)
    with pytest.raises(ValueError):
        pg.svdp(A, 3, which="XX", rng=np.random.default_rng(0))
    with pytest.raises(ValueError):
        pg.svdp(A, 3, which="SM", irl_mode=False, rng=np.random.default_rng(0))


def test_complex_input_is_fp64_only():
    """Complex input goes to the complex*16 drivers, which have no FP32 or
    mixed form: refused before any device work."""
    import numpy as np
    from scipy.sparse.linalg import LinearOperator
    import propack_gb300 as pg
    M = np.ones((6, 5)) + 1j * np.eye(6, 5)
    lo = LinearOperator(M.shape, matvec=lambda x: M @ x, rmatvec=lambda y: M.conj().T @ y, dtype=np.complex128)
    with pytest.raises(ValueError):
        pg.svdp(lo, 2, precision="mixed", rng=np.random.default_rng(0))


def _outcome(f):
    import propack_gb300 as pg
    try:
        f()
        return "ran"
    except ValueError:
        return "ValueError"
    except pg.PropackError:
        return "ran"  # validated, then no usable CUDA device on this host


@pytest.mark.parametrize("shifts", (None, -10, 0, 1, 10, 70))
def test_shifts_validation_matches_scipy(shifts):
    """The cases of scipy's test_propack.py::test_shifts: svdp refuses
    exactly the shifts scipy's _svdp refuses, before any device work."""
    import numpy as np
    from scipy.sparse.linalg import aslinearoperator
    from scipy.sparse.linalg._svdp import _svdp
    import propack_gb300 as pg
    n, k = 70, 10
    A = np.random.default_rng(0).random((n, n))
    ref = _outcome(lambda: _svdp(A, k, shifts=shifts, kmax=5 * k, irl_mode=True, rng=np.random.default_rng(0)))
    ours = _outcome(lambda: pg.svdp(aslinearoperator(A), k, shifts=shifts, kmax=5 * k, irl_mode=True,
                                    rng=np.random.default_rng(0)))
    assert ours == ref


@pytest.mark.parametrize("kw", [dict(k=0), dict(k=9), dict(k=3, kmax=2), dict(k=3, v0=np.ones(5)),
                                dict(k=3, which="SM", irl_mode=False), dict(k=3, which="XX")])
def test_argument_errors_match_scipy(kw):
    """k out of range, kmax < k, a start vector of the wrong length, 'SM'
    without restarts, an unknown `which`: the same ValueError as scipy."""
    from scipy.sparse.linalg import aslinearoperator
    from scipy.sparse.linalg._svdp import _svdp
    import propack_gb300 as pg
    A = np.random.default_rng(1).random((8, 6))
    kw = dict(kw)
    k = kw.pop("k")
    ref = _outcome(lambda: _svdp(A, k, rng=np.random.default_rng(0), **kw))
    ours = _outcome(lambda: pg.svdp(aslinearoperator(A), k, rng=np.random.default_rng(0), **kw))
    assert ref == "ValueError" and ours == ref


def test_process_wide_settings_refuse_bad_values():
    """The setters of the library's alternative kernels take only their
    documented values (checked on the host, no device work): the complex
    operator form, the restart products' tcgen05 kernel, the MLP layer's
    kernel, the batched arithmetic (and a batch handle that does not exist)."""
    import ctypes as C
    import propack_gb300 as pg
    L = pg.load()
    for fn, bad, good in (("propack_set_zcsr_form", (2, -1), 0), ("propack_set_gemm_impl", (0, 3), 2),
                          ("propack_mlp_set_impl", (2, -1), 1)):
        f = getattr(L, fn)
        f.restype = C.c_int
        f.argtypes = [C.c_int]
        for b in bad:
            assert f(b) == pg.ERR_ARG, (fn, b)
        assert f(good) == 0
    L.propack_batch_set_arith.restype = C.c_int
    L.propack_batch_set_arith.argtypes = [C.c_int64, C.c_int]
    assert L.propack_batch_set_arith(C.c_int64(123456789), 2) == pg.ERR_HANDLE
    assert L.propack_batch_set_arith(C.c_int64(123456789), 1) == pg.ERR_ARG
