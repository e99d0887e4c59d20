"""The differentiation form: binned forward pass against the CPU
restatement; the adjoint pass against the analytic gradient of the
accumulated per-bin coefficient sums and against central finite
differences (h = 1e-4); the torch.autograd.Function wrapper; a gradient fit
that recovers beta+ and |beta-|."""
import numpy as np
import pytest
import torch

from tp_autograd import log_likelihood

pytestmark = pytest.mark.gpu

SEED_DATA, SEED_MODEL = 777, 12345


@pytest.fixture(scope="module")
def setup(tp, ctx, cfg_sqrts1000):
    bins = tp.binning(20, 20)
    data_cfg = cfg_sqrts1000.replace(num_events=4_000_000, beta_plus=0.3, beta_minus=-0.2)
    data = ctx.binned_forward(data_cfg, 0, data_cfg.num_batches, bins, SEED_DATA)
    model_cfg = cfg_sqrts1000.replace(num_events=1_000_000, beta_plus=0.0, beta_minus=0.0)
    model = tp.BinnedGaussianLikelihood(ctx, model_cfg, SEED_MODEL, model_cfg.num_batches, data, data_cfg, bins)
    return bins, data_cfg, data, model_cfg, model


@pytest.mark.parametrize("ept", [40, 105, 313])
def test_binned_forward_matches_restatement(tp, oracle, cfg_sqrts1000, ept):
    """At 40 events per thread one batch fills a CTA; at 105 and 313 the CTA
    runs 2 and 8 batches at a time into its shared histogram."""
    cfg = cfg_sqrts1000.replace(num_events=200_000)
    bins = tp.binning(20, 20)
    with tp.Context(0) as ctx:
        ctx.set_events_per_thread(ept)
        gpu = ctx.binned_forward(cfg, 0, cfg.num_batches, bins, SEED_MODEL)
        # the binned total is the cross-section sum of the batch path
        acc = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", seed=SEED_MODEL)
    assert abs(gpu[:, 6].sum() - acc.sigma.sum()) <= 1e-12 * abs(acc.sigma.sum())
    e = cfg.e_total
    ref = oracle.binned(cfg, tp.rng_flags("xoshiro"), SEED_MODEL, 0, cfg.num_batches, 20, 20, (e / 3, e / 2),
                        (-cfg.beam_photons_cut, cfg.beam_photons_cut))
    assert np.array_equal(gpu[:, 5], ref[:, 5])  # events per bin
    k, _, _ = tp.coupling_factors(cfg)
    sc = np.array(oracle.sigma_contribs(cfg))
    sc_raw = k / sc  # per-contribution coupling factor (all sc != 0 off the Z peak)
    m_gpu = gpu[:, :5] * sc_raw
    tot = np.abs(ref[:, :5]).sum(axis=0)
    assert np.all(np.abs(m_gpu - ref[:, :5]).sum(axis=0) <= 1e-11 * tot)
    assert np.allclose(gpu[:, 6], ref[:, 6], rtol=1e-11, atol=1e-11 * np.abs(ref[:, 6]).max())
    assert np.allclose(gpu[:, 7], ref[:, 7], rtol=1e-11, atol=1e-11 * np.abs(ref[:, 7]).max())


@pytest.mark.parametrize("theta", [(0.0, 0.0, 91.187, 2.49), (0.25, -0.1, 91.187, 2.49), (1.0, 1.0, 91.0, 2.6)])
def test_adjoint_matches_analytic_gradient(setup, theta):
    _, _, _, _, model = setup
    lnl, grad, sigma, dsigma = model.gradient(theta)
    ga, dsa = model.analytic_gradient(theta)
    assert np.allclose(grad, ga, rtol=1e-10, atol=1e-10 * np.abs(ga).max())
    assert np.allclose(dsigma, dsa, rtol=1e-10, atol=1e-10 * np.abs(dsa).max())


def test_grad_entry_point(tp, setup):
    """tp_grad composes the adjoint sums with dK/dtheta in one call."""
    bins, _, _, _, model = setup
    theta = (0.25, -0.1, 91.187, 2.49)
    lnl, grad, sigma, dsigma = model.gradient(theta)
    cfg = model.theta_cfg(theta)
    _, _, mu = model.value(theta)
    r = -(mu - model.data) / model.var
    g, ds = model.ctx.grad(cfg, 0, model.n_batches, bins, r, model.seed, model.precision)
    assert np.allclose(g, grad, rtol=1e-13, atol=1e-13 * np.abs(grad).max())
    assert np.allclose(ds, dsigma, rtol=1e-13, atol=1e-13 * np.abs(dsigma).max())


def test_adjoint_matches_central_differences(setup):
    _, _, _, _, model = setup
    theta = np.array([0.25, -0.1, 91.187, 2.49])
    _, grad, _, dsigma = model.gradient(theta)
    for i in range(4):
        h = 1e-4 * max(abs(theta[i]), 1.0)
        tp_, tm = theta.copy(), theta.copy()
        tp_[i] += h
        tm[i] -= h
        lp, sp, _ = model.value(tp_)
        lm, sm, _ = model.value(tm)
        fd, fds = (lp - lm) / (2 * h), (sp - sm) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-5 * max(abs(grad[i]), 1e-3 * np.abs(grad).max()), (i, fd, grad[i])
        assert abs(fds - dsigma[i]) <= 1e-5 * max(abs(dsigma[i]), 1e-3 * np.abs(dsigma).max()), (i, fds, dsigma[i])


def test_adjoint_shape_invariance(tp, setup):
    """The adjoint sums do not depend on the block shape (events per thread):
    multi-warp CTAs at 40, one-warp CTAs at 313."""
    bins, _, _, _, model = setup
    theta = (0.25, -0.1, 91.187, 2.49)
    cfg = model.theta_cfg(theta)
    _, _, mu = model.value(theta)
    r = -(mu - model.data) / model.var
    out = []
    for ept in (40, 313):
        with tp.Context(0) as c:
            c.set_events_per_thread(ept)
            out.append(c.binned_adjoint(cfg, 0, model.n_batches, bins, r, model.seed, model.precision))
    (g1, s1), (g2, s2) = out
    assert np.allclose(g1, g2, rtol=1e-12, atol=1e-12 * np.abs(g1).max())
    assert np.allclose(s1, s2, rtol=1e-12, atol=1e-12 * np.abs(s1).max())


def test_fp32_adjoint_close_to_fp64(tp, setup):
    bins, data_cfg, data, model_cfg, model = setup
    m32 = tp.BinnedGaussianLikelihood(model.ctx, model_cfg, SEED_MODEL, model.n_batches, data, data_cfg, bins,
                                      precision=tp.TP_PREC_FP32_MIXED)
    theta = (0.25, -0.1, 91.187, 2.49)
    l64, g64, s64, ds64 = model.gradient(theta)
    l32, g32, s32, ds32 = m32.gradient(theta)
    assert abs(s32 - s64) <= 1e-6 * abs(s64)
    assert np.all(np.abs(g32 - g64) <= 1e-5 * np.abs(g64).max())


def test_torch_autograd_function(setup):
    _, _, _, _, model = setup
    theta = torch.tensor([0.25, -0.1, 91.187, 2.49], dtype=torch.float64, requires_grad=True)
    lnl = log_likelihood(theta, model)
    lnl.backward()
    _, grad, _, _ = model.gradient(theta.detach().tolist())
    assert torch.allclose(theta.grad, torch.tensor(grad), rtol=1e-12)


def test_gradient_fit_recovers_betas(tp, ctx, cfg_sqrts1000):
    # natural-gradient steps (adjoint gradient, Gauss-Newton Fisher
    # preconditioner) on (beta+, beta-) from near the model point beta+- = 0,
    # until a step moves both by less than 1e-3 of their errors.
    # Only beta-^2 enters the weights, so the data fix |beta-|; beta+ also
    # enters linearly through the interference terms.
    prec = tp.TP_PREC_FP32_MIXED
    bins = tp.binning(20, 20)
    data_cfg = cfg_sqrts1000.replace(num_events=20_000_000, beta_plus=0.3, beta_minus=-0.2)
    data = ctx.binned_forward(data_cfg, 0, data_cfg.num_batches, bins, SEED_DATA, prec)
    model_cfg = cfg_sqrts1000.replace(num_events=20_000_000, beta_plus=0.0, beta_minus=0.0)
    model = tp.BinnedGaussianLikelihood(ctx, model_cfg, SEED_MODEL, model_cfg.num_batches, data, data_cfg, bins,
                                        precision=prec)
    info = {}
    theta, cov = tp.fit(model, [0.05, 0.05, 91.187, 2.49], steps=200, lr=0.5, tol=1e-3, info=info)
    assert info["steps"] < 200
    err = np.sqrt(np.diag(cov))
    # statistical errors of data and model both enter (the likelihood only
    # counts the data's): allow 5 of the Fisher errors, at least 0.02
    tol = np.maximum(5 * np.sqrt(2) * err, 0.02)
    assert abs(theta[0] - 0.3) < tol[0] and abs(abs(theta[1]) - 0.2) < tol[1], (theta, err)
