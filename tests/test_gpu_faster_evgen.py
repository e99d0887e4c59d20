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


@pytest.mark.parametrize("rng,jump", [("ranf", False), ("xoshiro", False), ("ranf", True)])
def test_fp32_mixed_batch_range_equals_the_full_run(tp, ctx, cfg_valeurs, rng, jump):
    """FP32-mixed: a batch range inside the run gives the full run's batches
    bit for bit (its events, start states and per-batch sums do not depend
    on the range asked for)."""
    cfg = cfg_valeurs.replace(num_events=400_000)
    full = ctx.run_batches(cfg, 0, cfg.num_batches, rng=rng, jump_per_batch=jump, faster_evgen=True,
                           precision=tp.TP_PREC_FP32_MIXED)
    part = ctx.run_batches(cfg, 23, 9, rng=rng, jump_per_batch=jump, faster_evgen=True,
                           precision=tp.TP_PREC_FP32_MIXED)
    assert part.as_array().tobytes() == full.as_array()[23:32].tobytes()


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


@pytest.mark.parametrize("rng", ["xoshiro", "ranf"])
def test_without_the_bit_store(tp, oracle, ctx, cfg_valeurs, rng):
    """One-stream runs keep each chunk's accept bits, chases, walks and
    stream checkpoints between the map and starts passes; with the store
    off (tp_set_fe_store_cap(0), as for runs too large for it) the starts
    pass computes them again: identical batches, bit for bit, and the
    restatement's."""
    cfg = cfg_valeurs.replace(num_events=654_321)
    nb = cfg.num_batches
    kept = ctx.run_batches(cfg, 0, nb, rng=rng, faster_evgen=True)
    kept32 = ctx.run_batches(cfg, 0, nb, rng=rng, faster_evgen=True, precision=tp.TP_PREC_FP32_MIXED)
    ctx.set_fe_store_cap(0)
    try:
        again = ctx.run_batches(cfg, 0, nb, rng=rng, faster_evgen=True)
        again32 = ctx.run_batches(cfg, 0, nb, rng=rng, faster_evgen=True, precision=tp.TP_PREC_FP32_MIXED)
        part = ctx.run_batches(cfg, 17, 30, rng=rng, faster_evgen=True)
    finally:
        ctx.set_fe_store_cap(16 << 30)
    assert kept.as_array().tobytes() == again.as_array().tobytes()
    assert kept32.as_array().tobytes() == again32.as_array().tobytes()
    assert np.array_equal(kept32.selected, kept.selected)
    assert_batches_close(again, oracle_batches(tp, oracle, cfg, 0, nb, rng, False, True))
    assert_batches_close(part, oracle_batches(tp, oracle, cfg, 17, 30, rng, False, True))


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


@pytest.mark.parametrize("rng,jump", [("xoshiro", False), ("ranf", False), ("xoshiro", True), ("ranf", True)])
def test_fp32_mixed_selects_the_fp64_events(tp, ctx, cfg_sqrts1000, rng, jump):
    """The precision form of faster-evgen (the reference's fastest published
    mode is faster-evgen + f32): the same draws and accept decisions, FP32
    physics with the certified cut decisions, so the selected counts equal
    the FP64 run's batch by batch and the sums agree to FP32 accuracy."""
    cfg = cfg_sqrts1000.replace(num_events=1_000_000)
    nb = cfg.num_batches
    ctx.recheck_count(reset=True)
    f32 = ctx.run_batches(cfg, 0, nb, rng=rng, jump_per_batch=jump, precision=tp.TP_PREC_FP32_MIXED,
                          faster_evgen=True)
    rechecked = ctx.recheck_count(reset=True)
    f64 = ctx.run_batches(cfg, 0, nb, rng=rng, jump_per_batch=jump, faster_evgen=True)
    assert np.array_equal(f32.selected, f64.selected)
    assert 0 < rechecked < 1e-3 * cfg.num_events
    for name in ("sigma", "variance"):
        a, b = getattr(f32, name), getattr(f64, name)
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-5, name


@pytest.mark.parametrize("rng", ["xoshiro", "ranf"])
def test_fp32_mixed_res_data_within_1e6(tp, ctx, cfg_valeurs, rng):
    """res.data of a faster-evgen run at the reference's `valeurs` (1e7
    events) in FP32-mixed against FP64: the same selected events, every
    quantity within 1e-6 (the significances' uncertainties 1e-5, as for the
    default generator)."""
    r32 = tp.run_simulation(cfg_valeurs, rng=rng, precision=tp.TP_PREC_FP32_MIXED, ctx=ctx, faster_evgen=True)
    r64 = tp.run_simulation(cfg_valeurs, rng=rng, ctx=ctx, faster_evgen=True)
    assert r32.selected_events == r64.selected_events
    for f in ("sigma", "beta_min", "ss_p", "ss_m", "prec", "inc_ss_p", "inc_ss_m"):
        a, b = getattr(r32, f), getattr(r64, f)
        assert abs(a - b) <= (1e-5 if f.startswith("inc_") else 1e-6) * abs(b), (f, a, b)
    for s in range(2):
        for c in range(5):
            a, b = r32.spm2[s, c], r64.spm2[s, c]
            scale = abs(b) if c < 3 else max(abs(b), np.sqrt(abs(r64.spm2[s, 0] * r64.spm2[s, 1])))
            assert abs(a - b) <= 1e-6 * scale, (s, c, a, b)
