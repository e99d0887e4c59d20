"""Multi-process batch-range sharding (world size 2 and 3, gloo on CPU):
each rank integrates a contiguous batch range, the per-batch sums are
gathered once and merged in batch order, and the result equals the
single-process run bit for bit. The per-rank batch runner here is the CPU
restatement (no GPU in this test); on GPUs it is Context.run_batches."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_events, rng, jump, out_q):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]
    import torch.distributed as dist
    import __graft_entry__ as graft
    import tp_oracle_py

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    tp = graft.package()
    oracle = tp_oracle_py.Oracle(tp)
    _, cfg, _ = oracle.load(os.path.join(ROOT, "tests", "golden", "valeurs"))
    cfg = cfg.replace(num_events=n_events)
    kind = tp.rng_flags(rng, jump)

    def run_batches(first, n):
        return oracle.run_batches(cfg, first, n, kind, tp.default_seed(rng), threads=1)

    def all_gather(arr):
        got = [None] * world
        dist.all_gather_object(got, arr)
        return got

    res = tp.run_simulation_sharded(cfg, rank, world, run_batches, all_gather)
    if rank == 0:
        out_q.put(bytes(res.c))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,n_events,rng,jump", [(2, 53_000, "ranf", False), (2, 61_000, "xoshiro", True),
                                                     (3, 70_001, "xoshiro", False)])
def test_sharded_run_equals_single_process(tp, oracle, cfg_valeurs, world, n_events, rng, jump):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n_events, rng, jump, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    cfg = cfg_valeurs.replace(num_events=n_events)
    acc = oracle.run_batches(cfg, 0, cfg.num_batches, tp.rng_flags(rng, jump), tp.default_seed(rng))
    assert got == bytes(tp.merge_finalize(cfg, acc).c)
