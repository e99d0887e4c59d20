"""Batch-range sharding with the GPU as every rank's batch runner: ranks run
as host threads, each with its own context on the one GPU, and gather their
per-batch sums through the host (a barrier and a shared list; no kernel
waits on another). The merged result equals the single-context run bit for
bit. (The same function over gloo process groups is tested on the CPU.)"""
import threading

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("rng,jump", [("xoshiro", False), ("ranf", True)])
def test_gpu_shards_merge_to_the_single_run(tp, ctx, cfg_valeurs, world, rng, jump):
    cfg = cfg_valeurs.replace(num_events=345_678)
    slots = [None] * world
    results = [None] * world
    errors = []
    barrier = threading.Barrier(world, timeout=60)

    def rank_main(rank):
        try:
            with tp.Context(0) as c:
                def all_gather(arr):
                    slots[rank] = arr
                    barrier.wait()
                    return list(slots)

                run = lambda first, n: c.run_batches(cfg, first, n, rng=rng, jump_per_batch=jump)
                results[rank] = tp.run_simulation_sharded(cfg, rank, world, run, all_gather)
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(e)
            barrier.abort()

    threads = [threading.Thread(target=rank_main, args=(r,)) for r in range(world)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(120)
    assert not errors, errors
    whole = tp.run_simulation(cfg, rng=rng, jump_per_batch=jump, ctx=ctx)
    for r in results:
        assert bytes(r.c) == bytes(whole.c)
