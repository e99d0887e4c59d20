"""The differentiation form on the reference's default stream (ranf,
src/random/ranf.rs): binned forward pass against the CPU restatement
(one stream from draw 0 or per-batch reseeds, a range starting past batch
0), FP32-mixed bins equal to the FP64 ones, and the adjoint against the
analytic gradient of the forward pass's per-bin sums."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RANF_SEED = 234612947


def check_against_restatement(tp, oracle, cfg, gpu, kind, seed, first, n):
    e = cfg.e_total
    ref = oracle.binned(cfg, kind, seed, first, n, 20, 20, (e / 3, e / 2),
                        (-cfg.beam_photons_cut, cfg.beam_photons_cut))
    assert np.array_equal(gpu[:, 5], ref[:, 5])  # events per bin
    k, _, _ = tp.coupling_factors(cfg)
    sc_raw = k / np.array(oracle.sigma_contribs(cfg))
    m_gpu = gpu[:, :5] * sc_raw
    tot = np.abs(ref[:, :5]).sum(axis=0)
    assert np.all(np.abs(m_gpu - ref[:, :5]).sum(axis=0) <= 1e-11 * tot)
    assert np.allclose(gpu[:, 6], ref[:, 6], rtol=1e-11, atol=1e-11 * np.abs(ref[:, 6]).max())


@pytest.mark.parametrize("jump_per_batch,first", [(False, 0), (False, 7), (True, 3)])
def test_ranf_binned_forward_matches_restatement(tp, oracle, ctx, cfg_sqrts1000, jump_per_batch, first):
    cfg = cfg_sqrts1000.replace(num_events=205_000)  # ragged last batch
    n = cfg.num_batches - first
    bins = tp.binning(20, 20)
    gpu = ctx.binned_forward(cfg, first, n, bins, RANF_SEED, tp.TP_PREC_FP64, jump_per_batch, rng="ranf")
    kind = tp.rng_flags("ranf", jump_per_batch)
    check_against_restatement(tp, oracle, cfg, gpu, kind, RANF_SEED, first, n)
    # the binned total is the batch path's cross-section sum
    acc = ctx.run_batches(cfg, first, n, rng="ranf", seed=RANF_SEED, jump_per_batch=jump_per_batch)
    assert abs(gpu[:, 6].sum() - acc.sigma.sum()) <= 1e-12 * abs(acc.sigma.sum())


def test_ranf_fp32_bins_equal_fp64_bins(tp, ctx, cfg_sqrts1000):
    cfg = cfg_sqrts1000.replace(num_events=5_000_000)
    bins = tp.binning(20, 20)
    h32 = ctx.binned_forward(cfg, 0, cfg.num_batches, bins, RANF_SEED, tp.TP_PREC_FP32_MIXED, rng="ranf")
    h64 = ctx.binned_forward(cfg, 0, cfg.num_batches, bins, RANF_SEED, tp.TP_PREC_FP64, rng="ranf")
    assert np.array_equal(h32[:, 5], h64[:, 5])
    full = h64[:, 5] >= 1000
    for c in (0, 1, 2, 6):
        rel = np.abs(h32[:, c] - h64[:, c]) / np.abs(h64[:, c])
        assert rel[full].max() <= 1e-6, c


@pytest.fixture(scope="module")
def ranf_model(tp, ctx, cfg_sqrts1000):
    bins = tp.binning(20, 20)
    data_cfg = cfg_sqrts1000.replace(num_events=2_000_000, beta_plus=0.3, beta_minus=-0.2)
    data = ctx.binned_forward(data_cfg, 0, data_cfg.num_batches, bins, 1234567, rng="ranf")
    model_cfg = cfg_sqrts1000.replace(num_events=1_000_000, beta_plus=0.0, beta_minus=0.0)
    return tp.BinnedGaussianLikelihood(ctx, model_cfg, RANF_SEED, model_cfg.num_batches, data, data_cfg, bins,
                                       rng="ranf")


@pytest.mark.parametrize("theta", [(0.25, -0.1, 91.187, 2.49), (1.0, 1.0, 91.0, 2.6)])
def test_ranf_adjoint_matches_analytic_gradient(ranf_model, theta):
    lnl, grad, sigma, dsigma = ranf_model.gradient(theta)
    ga, dsa = ranf_model.analytic_gradient(theta)
    assert np.allclose(grad, ga, rtol=1e-10, atol=1e-10 * np.abs(ga).max())
    assert np.allclose(dsigma, dsa, rtol=1e-10, atol=1e-10 * np.abs(dsa).max())


def test_ranf_grad_entry_point_fp32(tp, ranf_model):
    """tp_grad on the ranf stream, FP32-mixed against FP64."""
    theta = (0.25, -0.1, 91.187, 2.49)
    cfg = ranf_model.theta_cfg(theta)
    _, _, mu = ranf_model.value(theta)
    r = -(mu - ranf_model.data) / ranf_model.var
    ctx, nb, bins = ranf_model.ctx, ranf_model.n_batches, ranf_model.bins
    g64, s64 = ctx.grad(cfg, 0, nb, bins, r, RANF_SEED, tp.TP_PREC_FP64, rng="ranf")
    g32, s32 = ctx.grad(cfg, 0, nb, bins, r, RANF_SEED, tp.TP_PREC_FP32_MIXED, rng="ranf")
    assert np.all(np.abs(g32 - g64) <= 1e-5 * np.abs(g64).max())
    assert np.all(np.abs(s32 - s64) <= 1e-6 * np.abs(s64).max())
