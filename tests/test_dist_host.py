"""Multi-process host logic of bench.py on CPU (gloo, world size 2): the
whole-job time is the slowest rank's, the rate counts every rank's units,
and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    mx = bench.max_over_ranks(10.0 * (rank + 1), ws)
    rate = bench.whole_job_rate(1000, 4, mx, ws)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(outdir, f"r{rank}.txt"), "w") as f:
        f.write(f"{mx} {rate}\n")


def test_max_over_ranks_and_whole_job_rate(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ws = 2
    mp.start_processes(_worker, args=(ws, _free_port(), str(tmp_path)), nprocs=ws, join=True, start_method="spawn")
    for r in range(ws):
        mx, rate = map(float, open(tmp_path / f"r{r}.txt").read().split())
        assert mx == 20.0
        assert abs(rate - 2 * 1000 * 4 / 0.020) < 1e-6


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        workload, steps, warmup, gpus = "c1", 1, 3, 2
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    bench.run_reference(A())  # returns without work on rank 1
    assert capsys.readouterr().out == ""
