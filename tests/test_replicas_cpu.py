"""Multi-GPU is replicas only (no data-path collective): the benchmark's job
time is the MAX over ranks and its value counts every rank's work.  Checked
with two gloo ranks on the CPU; the reference arm runs on rank 0 alone."""
import importlib.util
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    b = load_bench()
    local_ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    total_ms, value = b.replica_throughput(local_ms, 1e9, 4, world, dist, "cpu")
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"total_ms": total_ms, "value": value}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    for r in res:
        assert r["total_ms"] == 15.0
        # 2 ranks x 1 GFLOP x 4 steps in 15 ms
        assert r["value"] == pytest.approx(2 * 1e9 * 4 / 15e-3 / 1e12)


def test_single_rank_needs_no_process_group():
    b = load_bench()
    total_ms, value = b.replica_throughput(8.0, 2e9, 5, 1, None, "cpu")
    assert total_ms == 8.0 and value == pytest.approx(2e9 * 5 / 8e-3 / 1e12)


def test_reference_arm_prints_on_rank_zero_only():
    """Under torchrun every rank but 0 exits 0 without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
