"""The replica host path of bench.py with two gloo ranks on CPU: the process group,
the barrier, the max-over-ranks time, the whole-job rate and the rank-0-only reference
arm (the multi-GPU run is N independent replicas with no data-path collective)."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    w, r, local, dist = bench.dist_setup("gloo")
    assert (w, r, local) == (world, rank, rank) and dist is not None
    dist.barrier()
    t_ms = 10.0 * (rank + 1)  # rank 1 is the slow one
    t_max = bench.max_over_ranks(t_ms, dist)
    rate = bench.whole_job_rate(1000, w, 5, t_max)
    runs_ref = bench.reference_rank_runs(w, r)
    dist.barrier()
    with open(f"{out_path}.{rank}", "w") as f:
        f.write(f"{t_max} {rate} {int(runs_ref)}\n")
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    out = str(tmp_path / "res")
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    got = [open(f"{out}.{r}").read().split() for r in range(2)]
    for r, (t_max, rate, runs_ref) in enumerate(got):
        assert float(t_max) == 20.0                      # max over ranks
        assert float(rate) == pytest.approx(1000 * 2 * 5 / 0.020)
        assert int(runs_ref) == (1 if r == 0 else 0)     # reference arm on rank 0 alone


def test_single_process_defaults(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    w, r, local, dist = bench.dist_setup()
    assert (w, r, local, dist) == (1, 0, 0, None)
    assert bench.max_over_ranks(12.5, None) == 12.5
    assert bench.reference_rank_runs(1, 0)
