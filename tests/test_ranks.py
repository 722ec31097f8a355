"""The multi-rank logic of bench.py on host processes (gloo, world size 2).

One model's Newton iteration does not shard, so N GPUs run N independent
replicas: the ranks meet only at the barriers around the timed region and
in the reductions of the result (the slowest rank's time, the units of all
ranks).  These tests run that logic as two gloo ranks on the CPU, and the
reference arm's rule that only rank 0 works under torchrun.
"""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      CUDA_VISIBLE_DEVICES="4,6")    # the GPUs this job was given
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, torch, dist = bench.dist_setup()
    units = [100.0, 300.0][rank]          # replicas may differ in what they processed
    dt = [1.0, 2.0][rank]                 # and in how long they took
    res = {
        "world": w, "rank": r, "local": local, "backend": dist.get_backend(),
        "max": bench.max_over_ranks(rank + 1.5, w, torch, dist),
        "sum": bench.sum_over_ranks(rank + 1.5, w, torch, dist),
        "rate": bench.job_rate(units, dt, w, torch, dist),
        "visible": os.environ["CUDA_VISIBLE_DEVICES"],
    }
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(res, f)


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for rank in range(world):
        with open(tmp_path / f"rank{rank}.json") as f:
            res = json.load(f)
        assert res["world"] == world and res["rank"] == rank and res["local"] == rank
        assert res["backend"] == "gloo"
        assert res["max"] == 2.5                  # every rank sees the slowest time
        assert res["sum"] == 4.0
        assert res["rate"] == 400.0 / 2.0         # all units over the slowest rank's time
        assert res["visible"] == ["4", "6"][rank]  # its own GPU of the job's list


def test_single_rank_needs_no_process_group(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    world, rank, local, torch, dist = bench.dist_setup()
    assert (world, rank, local) == (1, 0, 0)
    assert not dist.is_initialized()
    assert bench.max_over_ranks(3.0, world, torch, dist) == 3.0
    assert bench.job_rate(10.0, 4.0, world, torch, dist) == 2.5


@pytest.mark.parametrize("arm", ["run_reference_frame", "run_reference_brick",
                                 "run_reference_batch", "run_reference_adjoint"])
def test_reference_arm_other_ranks_exit_without_work(monkeypatch, capsys, arm):
    # under torchrun rank 0 alone times the CPU path and prints its line; the
    # other ranks return 0 before touching their arguments
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    assert getattr(bench, arm)(None) is None
    assert capsys.readouterr().out == ""
