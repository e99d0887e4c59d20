"""`--features faster-evgen` on the GPU (TP_MODE_FASTER_EVGEN): rejection-
sampled unit-circle azimuths, 15 draws per event plus 2 per re-rolled point
(src/evgen.rs:143-173, 221-249), and ranf's random_array block skips
(src/random/ranf.rs:78-102).

The selected-event count of every batch is an exact check of every event
boundary: one misplaced draw shifts all later events of the stream and
changes the counts. Per-batch sums within 1e-12 of the CPU restatement,
res.data within 1e-12 of the reference's faster-evgen golden (N = 1e7)."""
import ctypes

import numpy as np
import pytest

from conftest import golden
from numdiff import compare
from test_gpu_parity import assert_batches_close

pytestmark = pytest.mark.gpu

MODES = [
    ("ranf", False, True),
    ("xoshiro", False, True),
    ("ranf", True, True),
    ("xoshiro", True, True),
    ("ranf", False, False),
]
IDS = ["ranf", "xoshiro", "ranf-jump", "xoshiro-jump", "ranf-nosort"]


def oracle_batches(tp, oracle, cfg, first, n, rng, jump, sort, seed=None):
    flags = tp.rng_flags(rng, jump, sort, faster_evgen=True)
    seed = tp.default_seed(rng) if seed is None else seed
    return oracle.run_batches(cfg, first, n, flags, seed)


@pytest.mark.parametrize("rng,jump,sort", MODES, ids=IDS)
def test_batches_match_restatement(tp, oracle, ctx, cfg_valeurs, rng, jump, sort):
    cfg = cfg_valeurs.replace(num_events=123_457)  # 13 batches, the last one partial
    nb = cfg.num_batches
    gpu = ctx.run_batches(cfg, 0, nb, rng=rng, jump_per_batch=jump, sorting=sort, faster_evgen=True)
    ref = oracle_batches(tp, oracle, cfg, 0, nb, rng, jump, sort)
    assert_batches_close(gpu, ref)


@pytest.mark.parametrize("rng,jump", [("ranf", False), ("xoshiro", False), ("xoshiro", True)])
def test_batch_range_inside_the_run(tp, oracle, ctx, cfg_valeurs, rng, jump):
    """first_batch > 0: the one-stream event boundaries are found from draw 0."""
    cfg = cfg_valeurs.replace(num_events=400_000)
    gpu = ctx.run_batches(cfg, 23, 9, rng=rng, jump_per_batch=jump, faster_evgen=True)
    ref = oracle_batches(tp, oracle, cfg, 23, 9, rng, jump, True)
    assert_batches_close(gpu, ref)
    # batches past the run are empty
    tail = ctx.run_batches(cfg, 38, 4, rng=rng, jump_per_batch=jump, faster_evgen=True)
    assert list(tail.selected[2:]) == [0, 0]
    assert_batches_close(tail, oracle_batches(tp, oracle, cfg, 38, 4, rng, jump, True))


@pytest.mark.parametrize("ept", [40, 64, 333, 10000])
def test_events_per_thread_invariance(tp, oracle, cfg_valeurs, ept):
    cfg = cfg_valeurs.replace(num_events=50_001)
    with tp.Context(0) as c:
        c.set_events_per_thread(ept)
        gpu = c.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", faster_evgen=True)
    assert_batches_close(gpu, oracle_batches(tp, oracle, cfg, 0, cfg.num_batches, "xoshiro", False, True))


def test_other_seeds(tp, oracle, ctx, cfg_sqrts1000):
    cfg = cfg_sqrts1000.replace(num_events=60_000)
    for rng, seed, jump in [("xoshiro", 2**63 + 17, False), ("ranf", 987654321, False), ("ranf", 2**31 - 5, True)]:
        gpu = ctx.run_batches(cfg, 0, cfg.num_batches, rng=rng, seed=seed, jump_per_batch=jump, faster_evgen=True)
        assert_batches_close(gpu, oracle_batches(tp, oracle, cfg, 0, cfg.num_batches, rng, jump, True, seed))


def test_golden_run(tp, ctx, cfg_valeurs):
    """The reference's faster-evgen golden: N = 1e7, ranf, one stream."""
    res = tp.run_simulation(cfg_valeurs, rng="ranf", faster_evgen=True, ctx=ctx)
    gold = golden("res.data", "faster-evgen")
    assert res.res_data().splitlines()[1] == gold.splitlines()[1]
    assert compare(res.res_data(), gold, rel_tol=1e-12) == []
    gold_out = golden("stdout.log", "faster-evgen")
    assert compare(res.report(), gold_out[gold_out.index("IBegin"):], rel_tol=1e-12) == []


def test_deterministic(ctx, cfg_valeurs):
    cfg = cfg_valeurs.replace(num_events=200_000)
    a = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", faster_evgen=True)
    b = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", faster_evgen=True)
    assert np.array_equal(a.selected, b.selected)
    assert a.as_array().tobytes() == b.as_array().tobytes()


def test_unsupported_combinations(tp, ctx, cfg_valeurs):
    cfg = cfg_valeurs.replace(num_events=10_000)
    with pytest.raises(tp.TPError) as e:
        ctx.run_batches(cfg, 0, 1, rng="xoshiro", precision=tp.TP_PREC_FP32_MIXED, faster_evgen=True)
    assert e.value.code == tp.TP_ERR_UNSUPPORTED
    flags = tp.rng_flags("xoshiro", faster_evgen=True)
    bins = tp.binning(4, 4)
    hist = np.zeros((16, tp.BIN_STRIDE), np.float64)
    st = tp.library().tp_binned_forward(ctx.h, ctypes.byref(cfg.c), flags, tp.XOSHIRO_DEFAULT_SEED, 0, 1,
                                        tp.TP_PREC_FP64, ctypes.byref(bins), ctypes.c_void_p(hist.ctypes.data))
    assert st == tp.TP_ERR_UNSUPPORTED
    dump = np.zeros(4, tp.DUMP_DTYPE)
    st = tp.library().tp_dump_events_prec(ctx.h, ctypes.byref(cfg.c), flags, tp.XOSHIRO_DEFAULT_SEED, 0, 4,
                                          tp.TP_PREC_FP64, ctypes.c_void_p(dump.ctypes.data))
    assert st == tp.TP_ERR_UNSUPPORTED
    # the context stays usable
    ctx.run_batches(cfg, 0, 1, rng="xoshiro", faster_evgen=True)


@pytest.mark.parametrize("seed", [42049, 176937])
def test_chunk_entered_past_the_mapped_offsets(tp, oracle, ctx, cfg_valeurs, seed):
    """Chunk maps cover entry offsets 0..31. These xoshiro seeds (found by
    simulating the stream on the CPU) have an event of more than 32 draws
    straddling a chunk boundary, so chunk 2 (seed 42049, entry 32) or chunk 3
    (seed 176937, entry 34) is entered past the mapped offsets and mapped
    again for its actual entry."""
    cfg = cfg_valeurs.replace(num_events=30_000)
    nb = cfg.num_batches
    gpu = ctx.run_batches(cfg, 0, nb, rng="xoshiro", seed=seed, faster_evgen=True)
    assert_batches_close(gpu, oracle_batches(tp, oracle, cfg, 0, nb, "xoshiro", False, True, seed))
