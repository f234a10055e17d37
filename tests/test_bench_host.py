"""Host-side pieces of bench.py on CPU: the reference arm's JSON line (its
keys, the two CPU baselines) on a small stand-in workload, and the
algorithmic-bytes formula of the SpMV roofline."""
import argparse
import json
import os

import pytest

import bench
from propack_gb300 import workloads


def test_reference_arm_json_contract(monkeypatch, capsys):
    small = workloads.zipf_mixed(seed=2, m=20000, hi=500)
    monkeypatch.setattr(bench, "make_workload", lambda name, scale=1.0: (small, None, None, None))
    args = argparse.Namespace(workload="zipf_mixed", steps=1, warmup=1, gpus=1, impl="reference", scale=1.0)
    assert bench.run_reference(args, bench.WORKLOADS["zipf_mixed"]) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "scipy_propack"):
        assert key in line, key
    assert line["impl"] == "reference" and line["higher_is_better"] is False
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    sc = line["scipy_propack"]
    assert "unavailable" in sc or (sc["value"] > 0 and sc["unit"] == "ms")


def test_spmv_bytes_formula():
    # values + int32 indices, row pointers, the gathered input, and three
    # passes over the output length (write y, read and write back prev)
    fwd, adj = bench.spmv_bytes(m=10, n=7, r=2, nnz_s=30, nnz_l=4, nnz_r=5, vb=8)
    assert fwd == 34 * 12 + 11 * 4 + 9 * 8 + 3 * 10 * 8
    assert adj == 35 * 12 + 8 * 4 + 12 * 8 + 3 * 7 * 8
    fwd32, _ = bench.spmv_bytes(m=10, n=7, r=0, nnz_s=30, nnz_l=0, nnz_r=0, vb=4)
    assert fwd32 == 30 * 8 + 11 * 4 + 7 * 4 + 3 * 10 * 4


@pytest.mark.parametrize("world", [1, 3])
def test_shards_cover_every_problem_once(world):
    costs = [5, 1, 3, 9, 9, 2, 7]
    got = sorted(i for r in range(world) for i in bench.shard_problems(costs, r, world))
    assert got == list(range(len(costs)))


@pytest.mark.parametrize("vis,local,want", [(None, 2, "2"), ("0,1,2,3", 2, "2"), ("4,5,6,7", 1, "5"),
                                            ("3", 1, "3"), ("", 0, "0")])
def test_each_rank_binds_its_own_gpu(monkeypatch, vis, local, want):
    """Under torchrun every rank takes its own device: its entry of a
    CUDA_VISIBLE_DEVICES list exported to all ranks, its local index when
    none is set, and a launcher's one-device binding as it is."""
    if vis is None:
        monkeypatch.delenv("CUDA_VISIBLE_DEVICES", raising=False)
    else:
        monkeypatch.setenv("CUDA_VISIBLE_DEVICES", vis)
    bench.bind_local_gpu(local)
    assert os.environ["CUDA_VISIBLE_DEVICES"] == want
