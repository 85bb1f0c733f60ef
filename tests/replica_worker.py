"""One rank of the two-rank ``gloo`` check of the bench's replica timing.

Kept apart from the test module so that spawned ranks import only this file
and ``bench`` (the package is registered under its import name by the test
session, not by a fresh interpreter)."""
import json
import os


def rank_main(rank, world, port, result_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = bench.max_over_ranks(10.0 + 7.5 * rank)        # rank 1 is the slow one
        val = bench.job_value(1000.0, 4, ms, world)
        with open(os.path.join(result_dir, f"r{rank}.json"), "w") as f:
            json.dump({"ms": ms, "value": val}, f)
    finally:
        dist.destroy_process_group()
