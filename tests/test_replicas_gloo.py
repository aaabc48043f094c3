"""CPU tests of the multi-rank (replica) path of bench.py with two gloo ranks: the barrier, the
max-over-ranks timing and the sum-over-ranks value behave as the bench contract needs (value =
units of all ranks / the slowest rank's time), and the reference arm prints on rank 0 only."""
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(world)
    t_max = bench.max_over_ranks(1.0 + rank, world)        # rank times 1.0 and 2.0 ms
    units = bench.sum_over_ranks(100.0 * (rank + 1), world)  # 100 and 200 units
    value = units / t_max
    bench.barrier(world)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"t_max": t_max, "units": units, "value": value}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_like_the_bench_contract(tmp_path):
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for r in res:
        assert r["t_max"] == 2.0 and r["units"] == 300.0 and r["value"] == 150.0


def _reference_rank(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world))
    import contextlib
    import io
    import bench
    buf = io.StringIO()
    sys.argv = ["bench.py", "--impl", "reference", "--workload", "tsmttsm-c1", "--steps", "1", "--warmup", "0"]
    with contextlib.redirect_stdout(buf):  # rank 0 runs the bounded CPU sample, rank 1 returns at once
        bench.main()
    with open(os.path.join(out_dir, f"ref{rank}.txt"), "w") as f:
        f.write(buf.getvalue())


def test_reference_arm_prints_on_rank_zero_only(tmp_path):
    from skinny_matmul_gb300 import build
    build.build()
    mp.start_processes(_reference_rank, args=(2, 0, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    out0 = (tmp_path / "ref0.txt").read_text().strip().splitlines()
    out1 = (tmp_path / "ref1.txt").read_text().strip()
    line = json.loads(out0[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["cores"] >= 1
    assert out1 == ""
