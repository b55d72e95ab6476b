"""The multi-rank host logic of bench.py on CPU: world-size-2 ``gloo`` process groups.

The step runs as independent replicas, one per GPU, with no collective on the data
path; the only exchange is the max over ranks of the timed step durations. These
tests run that exchange, the whole-job throughput built on it, and the reference
arm's rule that ranks other than 0 do no work, without a GPU.
"""
import json
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r's "durations": the slowest rank differs per entry
        mine = [10.0 + rank, 20.0 - rank, 5.0]
        got = bench.max_over_ranks(mine, "cpu")
        value = bench.replica_throughput(world, 4096 * 4096, got[0])
        dist.barrier()
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"max": got, "value": value}, f)


@pytest.mark.parametrize("world", [2, 3])
def test_max_over_ranks_gloo(tmp_path, world):
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    results = [json.loads((tmp_path / f"rank{r}.json").read_text()) for r in range(world)]
    want = [10.0 + world - 1, 20.0, 5.0]
    for r in results:
        assert r["max"] == want
        # whole-job throughput: all ranks' units over the slowest rank's time
        assert r["value"] == world * 4096 * 4096 / (want[0] * 1e-3)


def test_max_over_ranks_without_a_group():
    assert bench.max_over_ranks([1.5, 2], "cpu") == [1.5, 2.0]
    assert bench.replica_throughput(1, 1000, 2.0) == 1000 / 2e-3


def test_reference_arm_other_ranks_do_no_work(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = bench.argparse.Namespace(cpu_sample=8, steps=1, warmup=0, gpus=2)
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""
