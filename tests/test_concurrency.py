"""Reentrancy: the reference keeps its counters in COMMON blocks and SAVEs
state (double/stat.h, double/dsafescal.F:43), so it is not reentrant; here
every driver call has its own context and stream and the statistics are
per host thread.  Two host threads solving at once, each on its own
operator, must get the same bits as the same solves run one after the
other, and each thread's statistics must describe its own solve."""
import threading

import numpy as np
import pytest

import propack_gb300 as pg
from propack_gb300 import workloads

pytestmark = pytest.mark.gpu


def _problems():
    S1, L1, R1, w1 = workloads.lowrank_irl(seed=31, m=30000, n=8000, nnz_row=12, rank=10, udens=0.05, vdens=0.1)
    S2, L2, R2, w2 = workloads.lowrank_irl(seed=32, m=25000, n=12000, nnz_row=9, rank=6, udens=0.05, vdens=0.1)
    return [(S1, L1, R1, w1, 10), (S2, L2, R2, w2, 8)]


def _solve(op, k):
    u, s, vt, bnd = pg.svdp(op, k, irl_mode=True, kmax=3 * k, tol=1e-10, rng=np.random.default_rng(0))
    return u, s, vt, pg.get_stats()


def test_two_host_threads_give_the_serial_bits():
    probs = _problems()
    ops = [pg.CsrOperator(S, L, R, w) for S, L, R, w, _ in probs]
    ks = [p[-1] for p in probs]
    serial = [_solve(op, k) for op, k in zip(ops, ks)]
    out = [None, None]
    errors = []
    start = threading.Barrier(2)

    def worker(i):
        try:
            start.wait()
            out[i] = _solve(ops[i], ks[i])
        except Exception as e:  # reported below, on the main thread
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for i in range(2):
        u0, s0, vt0, st0 = serial[i]
        u1, s1, vt1, st1 = out[i]
        assert np.array_equal(s0, s1) and np.array_equal(u0, u1) and np.array_equal(vt0, vt1)
        assert st0["nopx"] == st1["nopx"] and st0["nrestart"] == st1["nrestart"]
    for op in ops:
        op.close()
