"""Batched form: many parameter points with uneven event counts in one
persistent launch (captured in a CUDA graph), against the one-point path on
the same streams, and the autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def batch_scale(b):
    """Per-element scale of (n, 12) batch sums (spm2[5], vars[5], sigma,
    variance): each sum's own size or its batch's A sum, and for the
    interference sums (which cancel) their natural size sqrt(|A| |B+|)."""
    scale = np.maximum(np.abs(b), np.abs(b[:, :1]))
    natural = np.sqrt(np.abs(b[:, 0] * b[:, 1]))
    scale[:, 3:5] = np.maximum(np.abs(b[:, 3:5]), natural[:, None])
    return scale


def small_points(tp, base, n=12, seed=5):
    cfgs, _ = tp.scan_points(base, n, seed)
    r = np.random.default_rng(seed)
    # uneven, ragged sizes: from one event to a few batches
    sizes = [1, 9999, 10000, 10001] + [int(x) for x in r.integers(1, 60_000, n - 4)]
    cfgs = [c.replace(num_events=s) for c, s in zip(cfgs, sizes)]
    seeds = [1000 + 7 * p for p in range(n)]
    starts = [tp.xoshiro_start(s) for s in seeds]
    return cfgs, seeds, starts


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32-mixed"])
def test_points_match_one_point_path(tp, cfg_valeurs, precision):
    cfgs, seeds, starts = small_points(tp, cfg_valeurs)
    with tp.Context(0) as ctx:
        parts = ctx.run_points(cfgs, starts, precision)
        again = ctx.run_points(cfgs, starts, precision)  # graph replay
        for cfg, seed, part, rep in zip(cfgs, seeds, parts, again):
            ref = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", seed=seed, precision=precision)
            # FP64: the tolerance of the batch tests; FP32-mixed: the two
            # kernels may contract FP32 products differently (the counts,
            # decided by the certified cuts, stay exact)
            tol = 1e-12 if precision == 0 else 1e-5
            for got in (part, rep):
                assert np.array_equal(got.selected, ref.selected)
                a, b = got.as_array()[:, 1:], ref.as_array()[:, 1:]
                assert np.all(np.abs(a - b) <= tol * np.maximum(batch_scale(b), 1e-300))
            assert rep.as_array().tobytes() == part.as_array().tobytes()  # graph replay is deterministic


def test_points_stream_is_jumped_seed(tp, oracle, cfg_sqrts1000):
    # scan_points' point p starts from seed 12345 jumped p times by 2^128
    # (the reference's faster-threading batch p), computed here by the
    # polynomial jump and by the restatement's matrix squaring
    _, starts = tp.scan_points(cfg_sqrts1000, 4)
    for p in range(4):
        assert [int(x) for x in starts[p]] == oracle.xoshiro_state(tp.XOSHIRO_DEFAULT_SEED, p)


def test_autotune_keeps_results(tp, cfg_sqrts1000):
    cfg = cfg_sqrts1000.replace(num_events=300_000)
    with tp.Context(0) as ctx:
        ref = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", precision=1)
        ept, rate = ctx.autotune(cfg, 1, 512)
        assert ept in (40, 53, 63, 79, 105, 157, 313) and rate > 1e9
        assert ctx.tuning(1)[0] == ept and ctx.tuning(1)[1] in (2, 3, 4)
        ctx.set_occupancy(0, 3)
        assert ctx.tuning(0) == (40, 3)  # FP64 keeps its own (default) shape
        got = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", precision=1)
    # the block shape regroups the per-thread FP32 sums: same events, sums
    # equal to FP32 accumulation accuracy
    assert np.array_equal(got.selected, ref.selected)
    assert np.allclose(got.sigma, ref.sigma, rtol=1e-6)


def test_scan_points_match_restatement(tp, oracle, cfg_sqrts1000):
    """Points of the benchmark's scan (random sqrt(s), E_min, cuts and
    beta+-, 1e6 to 1e8 events each) run by the persistent launch against
    the CPU restatement of the same point: its stream is seed 12345 jumped
    p times, consumed event after event across the point's batches. The
    first two batches and the last one of each point, FP64."""
    cfgs, starts = tp.scan_points(cfg_sqrts1000, 256, 12345)
    pick = [0, 1, 137]
    sub = [cfgs[p] for p in pick]
    with tp.Context(0) as ctx:
        parts = ctx.run_points(sub, starts[pick], 0)
    for p, cfg, part in zip(pick, sub, parts):
        nb = cfg.num_batches
        assert part.n == nb
        got = part.as_array()
        for b0, n in ((0, 2), (nb - 1, 1)):
            ref = oracle.run_batches_jumped(cfg, b0, n, tp.rng_flags("xoshiro"), tp.XOSHIRO_DEFAULT_SEED, p).as_array()
            a = got[b0:b0 + n]
            assert np.array_equal(a[:, 0], ref[:, 0]), (p, b0)
            scale = batch_scale(ref[:, 1:])
            assert np.all(np.abs(a[:, 1:] - ref[:, 1:]) <= 1e-12 * np.maximum(scale, 1e-300)), (p, b0)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32-mixed"])
def test_ranf_points_match_one_point_path(tp, cfg_valeurs, precision):
    """The batched form on the reference's default stream: point p is ranf
    seeded with its own seed, against tp_run_batches on that seed."""
    cfgs, _, _ = small_points(tp, cfg_valeurs)
    seeds = [tp.RANF_DEFAULT_SEED + 123456 * p for p in range(len(cfgs))]
    with tp.Context(0) as ctx:
        parts = ctx.run_points(cfgs, seeds, precision, rng="ranf")
        again = ctx.run_points(cfgs, seeds, precision, rng="ranf")  # graph replay
        for cfg, seed, part, rep in zip(cfgs, seeds, parts, again):
            ref = ctx.run_batches(cfg, 0, cfg.num_batches, rng="ranf", seed=seed, precision=precision)
            assert np.array_equal(part.selected, ref.selected)
            a, b = part.as_array()[:, 1:], ref.as_array()[:, 1:]
            # as for xoshiro: FP32 products may contract differently in the
            # two kernels; the counts (certified cuts) stay exact
            tol = 1e-12 if precision == 0 else 1e-5
            assert np.all(np.abs(a - b) <= tol * np.maximum(batch_scale(b), 1e-300))
            assert rep.as_array().tobytes() == part.as_array().tobytes()


def test_ranf_scan_points_match_restatement(tp, oracle, cfg_sqrts1000):
    """Points of the ranf scan (point p seeded 234612947 + 123456 p, the
    reference's p-th RandomGenerator::jump) against the CPU restatement of
    the same point, FP64: first two batches and the last one."""
    cfgs, seeds = tp.scan_points(cfg_sqrts1000, 256, 12345, rng="ranf")
    pick = [0, 3, 200]
    sub = [cfgs[p] for p in pick]
    with tp.Context(0) as ctx:
        parts = ctx.run_points(sub, seeds[pick], 0, rng="ranf")
    for p, cfg, part in zip(pick, sub, parts):
        nb = cfg.num_batches
        got = part.as_array()
        for b0, n in ((0, 2), (nb - 1, 1)):
            ref = oracle.run_batches_jumped(cfg, b0, n, tp.rng_flags("ranf"), tp.RANF_DEFAULT_SEED, p).as_array()
            a = got[b0:b0 + n]
            assert np.array_equal(a[:, 0], ref[:, 0]), (p, b0)
            scale = batch_scale(ref[:, 1:])
            assert np.all(np.abs(a[:, 1:] - ref[:, 1:]) <= 1e-12 * np.maximum(scale, 1e-300)), (p, b0)
