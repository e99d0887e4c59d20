"""K_c(theta) = couplings x sigma contributions and their derivatives in
theta = (beta+, beta-, M_Z, Gamma_Z) (host side, no GPU): values against
the restatement's constants, derivatives against central differences."""
import numpy as np
import pytest


@pytest.mark.parametrize("name", ["cfg_valeurs", "cfg_sqrts1000"])
def test_k_values(tp, oracle, request, name):
    cfg = request.getfixturevalue(name)
    k, dk, flux = tp.coupling_factors(cfg)
    g = oracle.couplings(cfg)
    sc = oracle.sigma_contribs(cfg)
    assert flux == 1.0 / (2.0 * cfg.e_total * cfg.e_total)
    # w = sum m_c sc_c with m_c = raw_c sc_raw_c: K_c / sc_c are the squared
    # coupling factors; their ratios are fixed by the couplings
    if sc[1] != 0 and sc[0] != 0:
        ratio = (k[1] / sc[1]) / (k[0] / sc[0])
        assert abs(ratio - (g[1] / g[0]) ** 2) <= 1e-13 * ratio


@pytest.mark.parametrize("name", ["cfg_valeurs", "cfg_sqrts1000"])
@pytest.mark.parametrize("theta0", [(1.0, 1.0), (0.3, -0.2), (0.0, 0.0)])
def test_k_derivatives_match_central_differences(tp, request, name, theta0):
    cfg = request.getfixturevalue(name).replace(beta_plus=theta0[0], beta_minus=theta0[1])
    k, dk, _ = tp.coupling_factors(cfg)
    fields = ["beta_plus", "beta_minus", "m_z0", "g_z0"]
    for i, f in enumerate(fields):
        x = getattr(cfg, f)
        def cd(h):
            kp, _, _ = tp.coupling_factors(cfg.replace(**{f: x + h}))
            km, _, _ = tp.coupling_factors(cfg.replace(**{f: x - h}))
            return (kp - km) / (2 * h)

        # Richardson-extrapolated central differences: O(h^4) truncation
        # (the Z-peak propagator is sharply curved in M_Z and Gamma_Z)
        h = 1e-4 * max(abs(x), 1.0)
        fd = (4 * cd(h / 2) - cd(h)) / 3
        scale = np.maximum(np.abs(k), 1e-300) / max(abs(x), 1.0)
        assert np.all(np.abs(fd - dk[:, i]) <= 1e-6 * np.maximum(np.abs(dk[:, i]), scale)), (f, fd, dk[:, i])
