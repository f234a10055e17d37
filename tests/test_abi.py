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


def test_kernels_compiled_for_sm103a():
    from propack_gb300 import _build
    lib = _build.build()
    out = subprocess.run(["cuobjdump", "--list-elf", lib], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


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
