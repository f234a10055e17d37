#!/usr/bin/env python
"""Benchmark: time to k converged singular triplets on one GB300.

Workload (default ``lowrank_irl``): DLANSVD_IRL in FP64 on a 2,000,000 x
500,000 sparse operator (20 N(0,1) nonzeros per row at uniform columns)
plus a rank-64 term sum_i 100*0.9^i u_i v_i' with sparse unit-norm u_i (1%
dense) and v_i (5% dense), kept factored; k = 50, Lanczos dimension 150
(p = 100 shifts), tol = 1e-10.  Seeded synthetic data (numpy default_rng(1)).

A step is one complete solve (start vector -> k converged Ritz triplets).

* value    device ms per solve with the operator already resident in HBM,
           from CUDA events the library records on the stream its kernels
           run on (start vector in HBM -> Ritz vectors in HBM).
* e2e      ms per solve through the public C ABI with HOST inputs: upload of
           the CSR arrays from pinned memory + device transpose + solve +
           copy of sigma, U(:,1:k), V(:,1:k) back to pinned memory.
* roofline the fused SpMV pair (the dominant HBM-bound kernel): algorithmic
           bytes per launch / mean launch time, from events around every
           launch in one profiled solve.
* cpu_baseline / --impl reference: the oracle (the C restatement of
           PROPACK with OpenMP) on the host cores, timing one complete IRL
           cycle (maxiter=1) of the same workload and scaling it to the
           matvec count of a full solve.

Inputs (operator ~1 GB, Lanczos basis 3 GB) are far larger than the 129 MB
L2, so no L2 flush is needed between steps.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "lowrank_irl": dict(
        desc="2000000x500000 CSR 20nnz/row N(0,1) + rank-64 sparse factored term (w_i=100*0.9^i), "
             "DLANSVD_IRL FP64 k=50 dim=150 p=100 tol=1e-10",
        k=50, kmax=150, tol=1e-10,
        # matvecs of a complete solve of this seeded workload, measured on GB300
        # (the GPU path and the oracle follow the same Lanczos trajectory);
        # used to scale the oracle's one-cycle sample to a full solve
        matvecs_full=1901,
    ),
}
# dram__bytes_read.sum + dram__bytes_write.sum per launch of the fused SpMV
# pair, from ncu on this workload (None until captured)
SPMV_TRAFFIC_BYTES = None


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="lowrank_irl", choices=sorted(WORKLOADS))
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="shrink m and n by this factor (profiling captures only; not a bench line)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(name, scale=1.0):
    from propack_gb300 import workloads
    if name == "lowrank_irl":
        return workloads.lowrank_irl(seed=1, m=int(2_000_000 * scale), n=int(500_000 * scale))
    raise ValueError(name)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        loaded = [s for s in sm if smax and s > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def spmv_bytes(m, n, r, nnz_s, nnz_l, nnz_r):
    """Algorithmic bytes of one fused SpMV launch, FP64 values / int32 indices:
    values+indices, row pointers, gathered input, written output, previous
    Lanczos vector read for the axpy and written back once scaled."""
    fwd = (nnz_s + nnz_l) * 12 + (m + 1) * 4 + (n + r) * 8 + 3 * m * 8
    adj = (nnz_s + nnz_r) * 12 + (n + 1) * 4 + (m + r) * 8 + 3 * n * 8
    return fwd, adj


def cpu_sample(S, L, R, w, wl, cores):
    """One complete IRL cycle of the oracle on the host cores, scaled to a full solve."""
    import numpy as np
    import oracle
    oracle.build()
    oracle.lib().oracle_set_threads(cores)
    op = oracle.Operator(S, L, R, w)
    oracle.clearstat()
    t0 = time.perf_counter()
    u, s, vt, bnd, info, kc = oracle.svdp(None, wl["k"], irl_mode=True, kmax=wl["kmax"], tol=wl["tol"],
                                          maxiter=1, rng=np.random.default_rng(0), op=op, compute_u=False,
                                          compute_v=False)
    dt = (time.perf_counter() - t0) * 1e3
    st = oracle.getstat()
    scale = wl["matvecs_full"] / max(st["nopx"], 1)
    return dt * scale, dict(cycle_ms=dt, cycle_matvecs=st["nopx"], scale=scale)


def run_reference(args, wl):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    S, L, R, w = make_workload(args.workload)
    vals = []
    for it in range(args.warmup + args.steps):
        v, info = cpu_sample(S, L, R, w, wl, cores)
        if it >= args.warmup:
            vals.append(v)
    value = statistics.mean(vals)
    sample = (f"oracle (C restatement of PROPACK dlansvd_irl, OpenMP) on {cores} host cores: one full IRL cycle "
              f"(maxiter=1: {info['cycle_matvecs']} matvecs, {info['cycle_ms']:.0f} ms) of the same workload, "
              f"scaled by matvecs to a full solve ({wl['matvecs_full']} matvecs)")
    line = {"impl": "reference", "metric": "ms to k=50 converged triplets (DLANSVD_IRL, resid<=1e-8*||A||)",
            "value": value, "unit": "ms", "higher_is_better": False, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "desc": wl["desc"]},
            "cpu_baseline": {"value": value, "unit": "ms", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(args, wl):
    rank, world, local = dist_env()
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    import numpy as np
    import propack_gb300 as pg
    pg.load()
    barrier = lambda: None
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        barrier = dist.barrier
    S, L, R, w = make_workload(args.workload, args.scale)
    m, n = S.shape
    r = L.shape[1]
    k, kmax, tol = wl["k"], wl["kmax"], wl["tol"]
    # reduced-scale runs only feed profiler captures: bound their restarts
    maxiter = 1000 if args.scale == 1.0 else 20

    def solve(op, u0=None):
        u = np.zeros((m, kmax + 1), order="F")
        v = np.zeros((n, kmax), order="F")
        sig, bnd = np.zeros(k), np.zeros(k)
        u[:, 0] = np.random.default_rng(0).uniform(size=m) if u0 is None else u0
        dop = np.array([np.sqrt(np.finfo(float).eps), np.finfo(float).eps ** 0.75, 0.0, 0.002])
        iop = np.array([0, 1], dtype=np.int32)
        kc, info = pg.lansvd_irl(b"L", b"y", b"y", m, n, kmax, kmax - k, k, maxiter, op.aprod, u, sig, bnd, v, tol,
                                 dop, iop, iparm=op.iparm)
        return kc, info, sig, u, v

    op = pg.CsrOperator(S, L, R, w)
    for _ in range(args.warmup):
        solve(op)
    sampler = ClockSampler(0) if rank == 0 else None
    if sampler:
        sampler.start()
    barrier()
    t0 = time.perf_counter()
    dev_ms, launches, matvecs, restarts = 0.0, 0, [], []
    for _ in range(args.steps):
        kc, info, sig, u, v = solve(op)
        st = pg.get_stats()
        dev_ms += st["solve_ms"]
        launches += st["kernel_launches"]
        matvecs.append(st["nopx"])
        restarts.append(st["nrestart"])
        if args.scale == 1.0:
            assert info == 0 and kc == k, (info, kc)
    wall_ms = (time.perf_counter() - t0) * 1e3
    barrier()
    clocks = sampler.stop() if sampler else None
    # residual check of the last solve (not timed): max ||A v - s u||, ||A' u - s v|| / ||A||
    res = 0.0
    for i in range(k):
        res = max(res, np.linalg.norm(op.matvec(v[:, i]) - sig[i] * u[:, i]),
                  np.linalg.norm(op.rmatvec(u[:, i]) - sig[i] * v[:, i]))
    rel_resid = res / sig[0]
    # per-kernel profile of one more solve (events around every launch)
    pg.set_profiling(True)
    solve(op)
    prof = pg.get_profile()
    pg.set_profiling(False)
    op.close()

    # e2e through the public API with pinned host buffers
    import torch
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    import scipy.sparse as sp
    h_parts = {}
    for nm, M in (("S", S), ("L", L), ("R", R)):
        M = sp.csr_array(M)
        h_parts[nm] = (pin(M.indptr.astype(np.int64)), pin(M.indices.astype(np.int32)), pin(M.data))
    h_w = pin(w)
    u_pin = torch.zeros((kmax + 1, m), dtype=torch.float64).pin_memory().numpy().T  # Fortran order
    v_pin = torch.zeros((kmax, n), dtype=torch.float64).pin_memory().numpy().T
    u0 = np.random.default_rng(0).uniform(size=m)
    e2e_steps = args.e2e_steps if args.e2e_steps is not None else max(1, min(args.steps, 2))

    class _Op:  # an operator built from the pinned host arrays through the C ABI
        pass

    lib = pg.load()
    import ctypes as C
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        h = C.c_int64(0)
        (sp_, si, sv), (lp, li, lv), (rp, ri, rv) = h_parts["S"], h_parts["L"], h_parts["R"]
        P = pg._i64p
        rc = lib.propack_csr_create(m, n, P(sp_), pg._ip(si), pg._dp(sv), r, P(lp), pg._ip(li), pg._dp(lv),
                                    P(rp), pg._ip(ri), pg._dp(rv), pg._dp(h_w), C.byref(h))
        assert rc == 0, pg.last_error()
        o = _Op()
        o.iparm = np.array([h.value & 0xFFFFFFFF, (h.value >> 32) & 0xFFFFFFFF], dtype=np.uint32).view(np.int32)
        o.aprod = C.cast(lib.propack_gpu_csr_aprod_, pg.APROD)
        u_pin[:, 0] = u0
        sig, bnd = np.zeros(k), np.zeros(k)
        dop = np.array([np.sqrt(np.finfo(float).eps), np.finfo(float).eps ** 0.75, 0.0, 0.002])
        iop = np.array([0, 1], dtype=np.int32)
        kc, info = pg.lansvd_irl(b"L", b"y", b"y", m, n, kmax, kmax - k, k, maxiter, o.aprod, u_pin, sig, bnd, v_pin,
                                 tol, dop, iop, iparm=o.iparm)
        if args.scale == 1.0:
            assert info == 0 and kc == k
        lib.propack_csr_destroy(h.value)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    barrier()
    h2d = sum(a.nbytes for t in h_parts.values() for a in t) + h_w.nbytes + m * 8
    d2h = 2 * k * 8 + k * (m + n) * 8

    # whole job: max over ranks
    total_dev = dev_ms
    if world > 1:
        import torch
        t = torch.tensor([total_dev, wall_ms, e2e_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_dev, wall_ms, e2e_ms = t.tolist()
    value = total_dev / (args.steps * world)

    if rank != 0:
        return 0
    fwd_b, adj_b = spmv_bytes(m, n, r, S.nnz, L.nnz, R.nnz)
    n_adj, t_adj = prof["spmv_adj"]
    n_fwd, t_fwd = prof["spmv_fwd"]
    achieved = (fwd_b * n_fwd + adj_b * n_adj) / ((t_fwd + t_adj) * 1e-3) / 1e9
    peak, peak_kind = peaks()
    roof = {"bound": "hbm", "kernel": "fused SpMV pair (k_lb_spmv<0>/<1>)", "achieved": achieved, "peak": peak,
            "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
            "traffic": SPMV_TRAFFIC_BYTES,
            "algorithmic_bytes_per_launch": {"fwd": fwd_b, "adj": adj_b},
            "mean_launch_ms": {"fwd": t_fwd / max(n_fwd, 1), "adj": t_adj / max(n_adj, 1)}}
    cpu = None
    if not args.no_cpu:
        cores = os.cpu_count() or 1
        cv, info = cpu_sample(S, L, R, w, wl, cores)
        cpu = {"value": cv, "unit": "ms", "cores": cores, "kind": "port",
               "sample": f"oracle one IRL cycle ({info['cycle_matvecs']} matvecs, {info['cycle_ms']:.0f} ms) "
                         f"scaled by matvecs to a full solve ({wl['matvecs_full']})"}
    breakdown = {kk: {"launches": c, "ms": t} for kk, (c, t) in prof.items() if c}
    line = {"metric": "ms to k=50 converged triplets (DLANSVD_IRL, resid<=1e-8*||A||)", "value": value,
            "unit": "ms", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": value,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded numpy default_rng(1))",
            "config": {"workload": args.workload, "desc": wl["desc"], "form": "plain FP64", "scale": args.scale,
                       "l2": "inputs larger than L2 (operator ~1 GB, basis ~3 GB); no flush"},
            "matvecs": statistics.mean(matvecs), "restarts": statistics.mean(restarts),
            "max_rel_residual": rel_resid, "wall_ms_per_step": wall_ms / args.steps,
            "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
            "kernel_breakdown": breakdown}
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)
    return run_ours(args, wl)


if __name__ == "__main__":
    sys.exit(main())
