"""FP32-mixed path against the FP64 path on the same events.

The cut decisions are certified: an event whose FP32 cut comparison lies
within the FP32 error bound is settled by an FP64 recheck, so the
selected-event counts must equal the FP64 path's exactly. The per-batch sums
carry FP32 rounding (about 1e-7 per event, averaging out); res.data
quantities must agree with the FP64 path within 1e-6 relative. The
interference (mixed) terms are compared on the larger of their own size and
their natural scale sqrt(|A| |B+|): they are statistically zero at
sqrt(s) = M_Z."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rng,jump", [("xoshiro", False), ("ranf", False), ("xoshiro", True), ("ranf", True)])
def test_fp32_decisions_match_fp64(tp, ctx, cfg_valeurs, rng, jump):
    cfg = cfg_valeurs.replace(num_events=1_000_000)
    nb = cfg.num_batches
    ctx.recheck_count(reset=True)
    f32 = ctx.run_batches(cfg, 0, nb, rng=rng, jump_per_batch=jump, precision=tp.TP_PREC_FP32_MIXED)
    rechecked = ctx.recheck_count(reset=True)
    f64 = ctx.run_batches(cfg, 0, nb, rng=rng, jump_per_batch=jump)
    assert np.array_equal(f32.selected, f64.selected)
    assert 0 < rechecked < 1e-3 * cfg.num_events
    # per-batch sums: FP32 events, FP64 batch sums
    for name in ("sigma", "variance"):
        a, b = getattr(f32, name), getattr(f64, name)
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-5, name
    for c in (0, 1, 2):
        assert np.max(np.abs(f32.spm2[c] - f64.spm2[c]) / np.abs(f64.spm2[c])) < 1e-5
        assert np.max(np.abs(f32.vars[c] - f64.vars[c]) / np.abs(f64.vars[c])) < 1e-5
    for c in (3, 4):
        scale = np.maximum(np.abs(f64.spm2[c]), np.sqrt(np.abs(f64.spm2[0] * f64.spm2[1])))
        assert np.max(np.abs(f32.spm2[c] - f64.spm2[c]) / scale) < 1e-5


@pytest.mark.parametrize("rng", ["xoshiro", "ranf"])
@pytest.mark.parametrize("cfg_name", ["cfg_valeurs", "cfg_sqrts1000"])
def test_fp32_res_data_within_1e6(tp, ctx, request, cfg_name, rng):
    """A systematic error in the FP32 draws adds up over the events instead
    of averaging out (ranf's n * fl(1e-9) moved A by 1.1e-6). The
    significances' uncertainties rest on the squared weights of a few heavy
    events, whose FP32 errors (up to 1e-5 each) average out more slowly:
    2e-6 at 1e7 events here, 1.4e-7 at 1e9."""
    cfg = request.getfixturevalue(cfg_name)
    cfg = cfg.replace(num_events=min(cfg.num_events, 10_000_000))
    r32 = tp.run_simulation(cfg, rng=rng, precision=tp.TP_PREC_FP32_MIXED, ctx=ctx)
    r64 = tp.run_simulation(cfg, rng=rng, ctx=ctx)
    assert r32.selected_events == r64.selected_events
    for f in ("sigma", "beta_min", "ss_p", "ss_m", "prec", "inc_ss_p", "inc_ss_m"):
        a, b = getattr(r32, f), getattr(r64, f)
        assert abs(a - b) <= (1e-5 if f.startswith("inc_") else 1e-6) * abs(b), (f, a, b)
    for s in range(2):
        for c in range(5):
            a, b = r32.spm2[s, c], r64.spm2[s, c]
            if c < 3:
                assert abs(a - b) <= 1e-6 * abs(b), (s, c, a, b)
            else:
                scale = max(abs(b), np.sqrt(abs(r64.spm2[s, 0] * r64.spm2[s, 1])))
                assert abs(a - b) <= 1e-6 * scale, (s, c, a, b)


def test_fp32_error_entry_point(tp, ctx, cfg_sqrts1000):
    """tp_fp32_error: the precision form's per-batch error against FP64 on
    the same events, for both streams."""
    cfg = cfg_sqrts1000.replace(num_events=300_000)
    for rng in ("xoshiro", "ranf"):
        err, a32, a64 = ctx.fp32_error(cfg, 0, cfg.num_batches, rng=rng)
        assert np.array_equal(a32.selected, a64.selected)
        # a batch's sums are dominated by a few heavy events, whose FP32
        # error reaches 1e-5; over the run the errors average out
        assert (err >= 0).all() and err.max() < 1e-4
        r32, r64 = tp.merge_finalize(cfg, a32), tp.merge_finalize(cfg, a64)
        assert abs(r32.sigma - r64.sigma) <= 1e-6 * abs(r64.sigma)
        ref64 = ctx.run_batches(cfg, 0, cfg.num_batches, rng=rng)
        assert a64.as_array().tobytes() == ref64.as_array().tobytes()
    # faster-evgen has its precision form too
    err = np.zeros(3)
    st = tp.library().tp_fp32_error(ctx.h, ctypes.byref(cfg.c), tp.rng_flags("xoshiro", faster_evgen=True), 1, 0, 3,
                                    err.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None, None)
    assert st == 0 and (err >= 0).all() and err.max() < 1e-4


def _headline_results(text):
    """sigma, its standard deviation and relative precision, beta_min and the
    B+- significances with their uncertainties: the res.data lines after the
    configuration echo (src/output.rs:62-142)."""
    import re
    out = []
    for line in text.splitlines()[17:26]:
        if ":" in line:
            out.extend(float(t) for t in re.findall(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?", line.split(":")[-1]))
    return np.array(out)


def test_fp32_mixed_against_the_reference_f32_build(tp, ctx, cfg_valeurs):
    """The reference's own all-FP32 build (`--features f32`) selects 1428
    events more than its FP64 build on the N = 1e7 standard-random golden run,
    and its res.data numbers move accordingly. The FP32-mixed path selects
    exactly the FP64 events and stays far closer to the FP64 golden on every
    number."""
    from conftest import golden

    res = tp.run_simulation(cfg_valeurs, rng="xoshiro", precision=tp.TP_PREC_FP32_MIXED, ctx=ctx)
    g64 = golden("res.data", "standard-random")
    g32 = golden("res.data", "standard-random,f32")
    assert res.res_data().splitlines()[1] == g64.splitlines()[1]
    assert g32.splitlines()[1] != g64.splitlines()[1]
    ours, ref64, ref32 = _headline_results(res.res_data()), _headline_results(g64), _headline_results(g32)
    assert ours.shape == ref64.shape == ref32.shape == (8,)
    err_ours = np.abs(ours - ref64) / np.abs(ref64)
    err_f32 = np.abs(ref32 - ref64) / np.abs(ref64)  # includes its 5-digit printing
    assert err_ours.max() < 1e-5
    # the f32 build's largest deviation (1.6e-3) is far above ours
    assert err_f32.max() > 100 * err_ours.max()


@pytest.mark.parametrize("rng", ["xoshiro", "ranf"])
def test_fp32_event_dumps(tp, ctx, cfg_sqrts1000, rng):
    """tp_dump_events_prec: the FP32-mixed path's view of single events
    (photons in energy order, as the reference lays them out) against the
    FP64 view of the same draws: the same cut verdicts, FP32-close momenta
    and helicity sums, and the rechecked events flagged."""
    n = 20_000
    d64 = ctx.dump_events(cfg_sqrts1000, 0, n, rng=rng)
    d32 = ctx.dump_events(cfg_sqrts1000, 0, n, rng=rng, precision=tp.TP_PREC_FP32_MIXED)
    assert np.array_equal(d32["uniforms"], d64["uniforms"])
    assert np.array_equal(d32["cut"], d64["cut"])
    assert d32["reserved"].sum() < 1e-3 * n and set(np.unique(d32["reserved"])) <= {0, 1}
    kept = d64["cut"] == 0
    assert 0.5 * n < kept.sum() < n
    # FP32 rounding of the raw momenta, amplified by the conformal map's
    # cancellation R_E^2 / R^2 (hundreds for a few events)
    dp = np.abs(d32["p_out"][kept] - d64["p_out"][kept]).max(axis=(1, 2)) / cfg_sqrts1000.e_total
    assert dp.max() < 2e-4 and np.median(dp) < 2e-7, (dp.max(), np.median(dp))
    for c in (0, 1, 2):
        a, b = d32["m2_sums"][kept, c], d64["m2_sums"][kept, c]
        rel = np.abs(a - b) / np.abs(b)
        assert rel.max() < 1e-3 and np.median(rel) < 1e-6, (c, rel.max(), np.median(rel))
