"""The multi-rank side of bench.py on CPU: two ranks over gloo (the search
has no exchange step, so ranks run independent replicas and meet only at
the timing barrier and the max-over-ranks reduction)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out_dir):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import torch
    import bench

    got_ws, got_rank, got_local = bench.dist_setup(None)
    bench.barrier(got_ws)
    # each rank's "step time": the job is as slow as its slowest rank
    ms = bench.max_over_ranks(got_ws, 10.0 + rank, torch, torch.device("cpu"))
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{got_ws} {got_rank} {got_local} {ms}\n")
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("the ranks would take NCCL on a GPU machine; this covers the CPU (gloo) side")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    rows = [open(tmp_path / f"rank{r}.txt").read().split() for r in range(2)]
    for r, (ws, rank, local, ms) in enumerate(rows):
        assert (int(ws), int(rank), int(local)) == (2, r, r)
        assert float(ms) == 11.0  # the max over both ranks on every rank


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.dist_setup(None) == (1, 0, 0)
    bench.barrier(1)
    assert bench.max_over_ranks(1, 3.5, None, None) == 3.5
