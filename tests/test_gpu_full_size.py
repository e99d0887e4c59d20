"""Parity at the benchmark configurations' full sizes: 1e9 events (1e5
batches, 1.2e10 draws) and 1e10 events (1e6 batches, 1.2e11 draws), where
the CPU restatement cannot run every event.

- The last batches of each run against the restatement, which reaches them
  by its own jump-ahead (powers of the generators' transition matrices),
  not the product's characteristic-polynomial method.
- Size-independent properties of a whole 1e9-event run: the per-batch sums
  do not depend on how the batch range is split into calls (bit for bit),
  and the FP32-mixed path selects exactly the FP64 path's events in every
  batch."""
import numpy as np
import pytest

from test_gpu_parity import assert_batches_close, rel

pytestmark = pytest.mark.gpu

N1, N2 = 1_000_000_000, 10_000_000_000


@pytest.mark.parametrize("rng", ["xoshiro", "ranf"])
def test_config1_last_batches(tp, oracle, ctx, cfg_sqrts1000, rng):
    cfg = cfg_sqrts1000.replace(num_events=N1)
    first, n = cfg.num_batches - 6, 6
    gpu = ctx.run_batches(cfg, first, n, rng=rng)
    ref = oracle.run_batches(cfg, first, n, tp.rng_flags(rng), tp.default_seed(rng))
    assert_batches_close(gpu, ref)


@pytest.mark.parametrize("rng", ["xoshiro", "ranf"])
def test_config2_last_batches(tp, oracle, ctx, cfg_sqrts1000, rng):
    cfg = cfg_sqrts1000.replace(num_events=N2)
    first, n = cfg.num_batches - 4, 4
    ref = oracle.run_batches(cfg, first, n, tp.rng_flags(rng), tp.default_seed(rng))
    gpu64 = ctx.run_batches(cfg, first, n, rng=rng)
    assert_batches_close(gpu64, ref)
    gpu32 = ctx.run_batches(cfg, first, n, rng=rng, precision=tp.TP_PREC_FP32_MIXED)
    assert np.array_equal(gpu32.selected, ref.selected)
    assert rel(gpu32.sigma, ref.sigma) < 1e-6


@pytest.fixture(scope="module")
def full_run(tp, cfg_sqrts1000):
    cfg = cfg_sqrts1000.replace(num_events=N1)
    with tp.Context(0) as c:
        whole = c.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro")
    return cfg, whole


def test_full_run_split_invariance(tp, full_run):
    cfg, whole = full_run
    nb = cfg.num_batches
    cuts = [0, 1, 33_333, 65_536, 70_001, nb]
    with tp.Context(0) as c:
        parts = [c.run_batches(cfg, a, b - a, rng="xoshiro") for a, b in zip(cuts[:-1], cuts[1:])]
    joined = np.concatenate([p.as_array() for p in parts], axis=0)
    assert joined.tobytes() == whole.as_array().tobytes()


def test_full_run_fp32_selects_the_fp64_events(tp, full_run):
    cfg, whole = full_run
    with tp.Context(0) as c:
        fp32 = c.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", precision=tp.TP_PREC_FP32_MIXED)
    assert np.array_equal(fp32.selected, whole.selected)
    a = tp.merge_finalize(cfg, whole)
    b = tp.merge_finalize(cfg, fp32)
    assert abs(b.sigma - a.sigma) <= 1e-6 * abs(a.sigma)


@pytest.mark.parametrize("rng", ["xoshiro", "ranf"])
def test_batches_2_to_the_40_in(tp, oracle, ctx, cfg_sqrts1000, rng):
    """Batches around index 2^40 of a 2^40 + 8 batch run (1.3e17 draws in):
    64-bit draw offsets far past the benchmark sizes, against the oracle's
    transition-matrix powers; FP32-mixed selects the same events."""
    first = 2**40 - 2
    cfg = cfg_sqrts1000.replace(num_events=(2**40 + 8) * tp.TP_BATCH_SIZE)
    ref = oracle.run_batches(cfg, first, 4, tp.rng_flags(rng), tp.default_seed(rng))
    assert_batches_close(ctx.run_batches(cfg, first, 4, rng=rng), ref)
    gpu32 = ctx.run_batches(cfg, first, 4, rng=rng, precision=tp.TP_PREC_FP32_MIXED)
    assert np.array_equal(gpu32.selected, ref.selected)
