"""bench.py host logic: byte model, workload definitions, replica aggregation over 2 gloo ranks (CPU),
and the CPU reference arm's JSON line."""
import json
import os
import subprocess
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bytes_model():
    assert bench.bytes_model(10, 100, 8) == 10 * 32 + 100 * 16
    assert bench.bytes_model(10, 100, 16) == 10 * 48 + 100 * 24


def test_workload_bond_counts():
    n, bonds, jxy, jz, shape, k = bench.hamiltonian_spec(bench.WORKLOADS["chain24_k0"])
    assert (n, len(bonds), shape) == (24, 24, (24, 1))
    n, bonds, jxy, jz, shape, k = bench.hamiltonian_spec(bench.WORKLOADS["square6x6_k0"])
    assert (n, len(bonds), shape) == (36, 144, (6, 6))
    assert sorted(set(jxy)) == [0.5, 1.0]
    assert len(set(map(tuple, map(sorted, bonds)))) == 144


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t, b = bench.combine_ranks(0.5 + rank, 100.0 * (rank + 1))
    dist.destroy_process_group()
    q.put((rank, t, b))


def test_combine_ranks_gloo_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert all(abs(t - 1.5) < 1e-12 and abs(b - 300.0) < 1e-9 for _, t, b in res)


def test_reference_arm_prints_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "chain16_full", "--steps", "5", "--warmup", "3"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"):
        assert key in line
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_bench_options_parse_without_gpu():
    """The bench's command line (slab variants and layouts, batch launch modes) parses on the CPU."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                       cwd=ROOT, timeout=120)
    assert r.returncode == 0, r.stderr
    for opt in ("--slab-mode", "--slab-scaling", "--slab-mb", "--batch-launch", "--workload"):
        assert opt in r.stdout
    assert "four lanes per row" in r.stdout
