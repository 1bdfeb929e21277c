"""The multi-rank parts of bench.py on the CPU, as world-size-2 gloo process groups: the rank environment,
the whole-job aggregation (units summed over ranks, the slowest rank's time), and the reference arm's ranks
other than 0 exiting without work.  One process per rank, started with `spawn`."""
import json
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    sys.path.insert(0, str(ROOT))
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    import torch.distributed as dist

    import bench
    w, r, local = bench.dist_setup()
    dist.init_process_group("gloo", rank=r, world_size=w)
    # rank r traced 100 (r + 1) units in 10 + r ms
    units, ms = bench.aggregate(100.0 * (r + 1), 10.0 + r, w, "cpu")
    dist.barrier()
    dist.destroy_process_group()
    Path(out_dir, f"rank{r}.json").write_text(json.dumps({"env": [w, r, local], "units": units, "ms": ms}))


def test_aggregate_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn",
                       join=True)
    for r in range(world):
        res = json.loads((tmp_path / f"rank{r}.json").read_text())
        assert res["env"] == [world, r, r]
        assert res["units"] == 300.0  # 100 + 200: the whole job's work
        assert res["ms"] == 11.0  # the slowest rank


def test_single_rank_aggregate_is_the_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.aggregate(123.0, 4.5, 1) == (123.0, 4.5)


def test_reference_arm_other_ranks_do_no_work(capsys):
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.run_reference(None, 2, 1) is None  # returns before reading its arguments
    assert capsys.readouterr().out == ""
