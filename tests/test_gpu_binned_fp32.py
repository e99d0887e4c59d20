"""The FP32-mixed binned passes bin every event where the FP64 pass does:
the bin decision is certified like the cut decisions (an event whose FP32
energy or cosine lies within its error bound of an inner bin edge, or whose
two leading photons are within their errors of each other, is binned from
FP64 momenta). Per-bin event counts equal the FP64 pass's exactly; per-bin
sums agree to FP32 accuracy; the adjoint sees the same bins."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed,betas", [(12345, (0.0, 0.0)), (777, (0.3, -0.2))])
def test_fp32_bins_equal_fp64_bins(tp, ctx, cfg_sqrts1000, seed, betas):
    cfg = cfg_sqrts1000.replace(num_events=10_000_000, beta_plus=betas[0], beta_minus=betas[1])
    bins = tp.binning(20, 20)
    ctx.recheck_count(reset=True)
    h32 = ctx.binned_forward(cfg, 0, cfg.num_batches, bins, seed, tp.TP_PREC_FP32_MIXED)
    settled = ctx.recheck_count(reset=True)
    h64 = ctx.binned_forward(cfg, 0, cfg.num_batches, bins, seed, tp.TP_PREC_FP64)
    assert np.array_equal(h32[:, 5], h64[:, 5]), np.flatnonzero(h32[:, 5] != h64[:, 5])
    # FP32 per-event values summed per bin: within 1e-6 of each bin's own
    # sum wherever a bin holds 1000 events or more (single events carry FP32
    # errors up to 1e-4 in their B+- sums, which sparse edge bins do not
    # average away: 1e-4 there); the interference sums, which cancel, on
    # their natural scale sqrt(|A| |B+|) in the bin
    full = h64[:, 5] >= 1000
    natural = np.sqrt(np.abs(h64[:, 0] * h64[:, 1]))
    for c in range(8):
        scale = np.abs(h64[:, c]) if c not in (3, 4) else np.maximum(np.abs(h64[:, c]), natural)
        rel = np.abs(h32[:, c] - h64[:, c]) / np.maximum(scale, 1e-300)
        print("sum %d: max rel. error %.2e over full bins, %.2e over all" % (c, rel[full].max(), rel.max()))
        assert rel[full].max() <= 1e-6 and rel.max() <= 1e-4, c
    # some events needed the FP64 decision (cuts or bins), a small fraction
    assert 0 < settled < 0.01 * cfg.num_events


def test_fp32_bins_other_shapes(tp, cfg_sqrts1000):
    """Finer bins, an explicit range and another block shape (40 events per
    thread: one batch per 256-thread CTA)."""
    cfg = cfg_sqrts1000.replace(num_events=2_000_000)
    bins = tp.binning(32, 32, emax=(340.0, 495.0), cos=(-0.9, 0.9))
    with tp.Context(0) as c:
        c.set_events_per_thread(40)
        h32 = c.binned_forward(cfg, 0, cfg.num_batches, bins, 4242, tp.TP_PREC_FP32_MIXED)
        h64 = c.binned_forward(cfg, 0, cfg.num_batches, bins, 4242, tp.TP_PREC_FP64)
    assert np.array_equal(h32[:, 5], h64[:, 5])


def test_fp32_adjoint_uses_fp64_bins(tp, ctx, cfg_sqrts1000):
    """With a bin weight that is 1 in one bin and 0 elsewhere, the adjoint's
    sum of raw_0 is that bin's raw_0 sum of the FP64 forward pass."""
    cfg = cfg_sqrts1000.replace(num_events=2_000_000)
    bins = tp.binning(20, 20)
    h64 = ctx.binned_forward(cfg, 0, cfg.num_batches, bins, 99, tp.TP_PREC_FP64)
    for b in (0, 57, 210):
        r = np.zeros(400)
        r[b] = 1.0
        g, s = ctx.binned_adjoint(cfg, 0, cfg.num_batches, bins, r, 99, tp.TP_PREC_FP32_MIXED)
        assert abs(g[0] - h64[b, 0]) <= 1e-6 * abs(h64[b, 0]), (b, g[0], h64[b, 0])
