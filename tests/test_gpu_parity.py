"""GPU event loop (through the C ABI) against the CPU restatement and the
reference's goldens.

Integer results (uniforms, cut decisions, selected-event counts) must be
bit-exact. Floating-point sums: per batch within 1e-12 relative (the GPU
sums a batch in a tree, the reference left to right; measured differences
are ~1e-15). Momenta: within 64 ulps (CUDA's log/sin/cos and glibc's may
differ in their last bit)."""
import ctypes

import numpy as np
import pytest

from conftest import golden
from numdiff import compare

pytestmark = pytest.mark.gpu

MODES = [
    ("ranf", False, True),
    ("xoshiro", False, True),
    ("ranf", True, True),
    ("xoshiro", True, True),
    ("ranf", False, False),
    ("xoshiro", False, False),
]
IDS = ["ranf", "xoshiro", "ranf-jump", "xoshiro-jump", "ranf-nosort", "xoshiro-nosort"]


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0


def assert_batches_close(gpu, ref, tol=1e-12):
    assert np.array_equal(gpu.selected, ref.selected)
    for name in ("spm2", "vars", "sigma", "variance"):
        g, r = getattr(gpu, name), getattr(ref, name)
        if name in ("spm2",):
            # Re/Im(mixed) sums cancel: compare them on the scale of the A row
            scale = np.maximum(np.abs(r), np.abs(ref.spm2[0])[None, :])
            err = float(np.max(np.abs(g - r) / np.maximum(scale, 1e-300)))
        else:
            err = rel(g, r)
        assert err < tol, (name, err)


@pytest.mark.parametrize("rng,jump,sort", MODES, ids=IDS)
def test_batches_match_restatement(tp, oracle, ctx, cfg_valeurs, rng, jump, sort):
    cfg = cfg_valeurs.replace(num_events=123_456)  # 13 batches, the last one partial
    nb = cfg.num_batches
    gpu = ctx.run_batches(cfg, 0, nb, rng=rng, jump_per_batch=jump, sorting=sort)
    ref = oracle.run_batches(cfg, 0, nb, tp.rng_flags(rng, jump, sort), tp.default_seed(rng))
    assert_batches_close(gpu, ref)
    assert gpu.selected[-1] < gpu.selected[0]  # partial batch


@pytest.mark.parametrize("rng,jump", [("ranf", False), ("xoshiro", False), ("xoshiro", True), ("ranf", True)])
def test_resume_at_any_batch(tp, oracle, ctx, cfg_valeurs, rng, jump):
    # batch b's stream is a pure function of b: resuming at batch 977 of a
    # 1e7 run gives the same accumulators as the uninterrupted run
    cfg = cfg_valeurs
    gpu = ctx.run_batches(cfg, 977, 3, rng=rng, jump_per_batch=jump)
    ref = oracle.run_batches(cfg, 977, 3, tp.rng_flags(rng, jump), tp.default_seed(rng))
    assert_batches_close(gpu, ref)


@pytest.mark.parametrize("n", [1, 7, 9999, 10000, 10001, 20000])
def test_small_and_ragged_sizes(tp, oracle, ctx, cfg_valeurs, n):
    cfg = cfg_valeurs.replace(num_events=n)
    for rng in ("ranf", "xoshiro"):
        gpu = ctx.run_batches(cfg, 0, cfg.num_batches, rng=rng)
        ref = oracle.run_batches(cfg, 0, cfg.num_batches, tp.rng_flags(rng), tp.default_seed(rng))
        assert_batches_close(gpu, ref)


def test_batches_beyond_the_run_are_empty(tp, ctx, cfg_valeurs):
    cfg = cfg_valeurs.replace(num_events=25_000)
    gpu = ctx.run_batches(cfg, 0, 5, rng="xoshiro")
    assert gpu.selected[3] == 0 and gpu.selected[4] == 0 and gpu.sigma[4] == 0.0


@pytest.mark.parametrize("rng,jump,sort", MODES[:4], ids=IDS[:4])
def test_event_dumps(tp, oracle, ctx, cfg_valeurs, rng, jump, sort):
    first, n = 9_990_000 - 37, 20_000  # crosses a batch boundary
    g = ctx.dump_events(cfg_valeurs, first, n, rng=rng, jump_per_batch=jump, sorting=sort)
    r = oracle.dump_events(cfg_valeurs, tp.rng_flags(rng, jump, sort), tp.default_seed(rng), first, n)
    assert np.array_equal(g["uniforms"], r["uniforms"])  # bit-exact draws
    assert np.array_equal(g["cut"], r["cut"])  # identical cut decisions
    # momenta within 1e-12 of sqrt(s): CUDA's and glibc's log/sin/cos may
    # differ in their last bit, which the conformal map amplifies when the
    # three raw photons are nearly collinear (R^2 = R_E^2 - |R|^2 cancels)
    d = np.abs(g["p_out"] - r["p_out"])
    assert float(d.max()) <= 1e-12 * cfg_valeurs.e_total, float(d.max())
    ulp = np.spacing(np.abs(r["p_out"]).max(axis=2, keepdims=True))
    assert np.mean(d <= 8 * ulp) > 0.99
    kept = r["cut"] == 0
    m_g, m_r = g["m2_sums"][kept], r["m2_sums"][kept]
    # amplitude algebra: the GPU's m2 against the restatement's formulas
    # evaluated on the GPU's own momenta
    m_same = oracle.m2_sums_of(cfg_valeurs, g["p_out"][kept][:2000])
    scale = np.maximum(np.abs(m_same), np.abs(m_same[:, :1]))
    alg = np.abs(m_g[:2000] - m_same) / scale
    # photons close to the -z axis (xx = sqrt(E + Z) cancels) amplify the
    # rounding differences of two equivalent formulas
    assert np.max(alg) < 1e-10 and np.quantile(alg, 0.99) < 1e-13
    # end to end: bounded by the conditioning of the momenta (above)
    scale = np.maximum(np.abs(m_r), np.abs(m_r[:, :1]))
    err = np.abs(m_g - m_r) / scale
    assert np.max(err) < 1e-9 and np.median(err) < 1e-14


@pytest.mark.parametrize("features,rng,jump,sort", [
    ("", "ranf", False, True),
    ("standard-random", "xoshiro", False, True),
    ("multi-threading,faster-threading", "ranf", True, True),
    ("standard-random,multi-threading,faster-threading", "xoshiro", True, True),
    ("no-photon-sorting", "ranf", False, False),
])
def test_golden_run(tp, ctx, cfg_valeurs, features, rng, jump, sort):
    res = tp.run_simulation(cfg_valeurs, rng=rng, jump_per_batch=jump, sorting=sort, ctx=ctx)
    gold = golden("res.data", features)
    # the selected-event count is an exact check of every cut decision
    assert res.res_data().splitlines()[1] == gold.splitlines()[1]
    assert compare(res.res_data(), gold, rel_tol=1e-12) == []
    gold_out = golden("stdout.log", features)
    assert compare(res.report(), gold_out[gold_out.index("IBegin"):], rel_tol=1e-12) == []


@pytest.mark.parametrize("cfg_name", ["cfg_valeurs", "cfg_sqrts1000"])
def test_photon_order_symmetry(tp, ctx, request, cfg_name):
    """Without the plane cut the cuts and the helicity sums are symmetric
    under permutations of the photons: sorted and unsorted runs select the
    same events and agree to rounding (the FP32-mixed kernels rely on it and
    leave the photons unsorted)."""
    cfg = request.getfixturevalue(cfg_name).replace(num_events=200_000)
    assert cfg.beam_photon_plane_cut <= 0.0
    a = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro")
    b = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", sorting=False)
    assert_batches_close(a, b, tol=1e-13)


def test_deterministic(ctx, cfg_valeurs):
    cfg = cfg_valeurs.replace(num_events=200_000)
    a = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro")
    b = ctx.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro")
    assert a.as_array().tobytes() == b.as_array().tobytes()


@pytest.mark.parametrize("ept", [80, 313])
@pytest.mark.parametrize("precision,occ", [(0, 2), (0, 3), (1, 2), (1, 3), (1, 4)])
def test_kernel_variants(tp, oracle, cfg_valeurs, precision, occ, ept):
    """The register/occupancy variants of the xoshiro event kernels, in
    multi-warp (80 events per thread) and one-warp (313) CTAs."""
    cfg = cfg_valeurs.replace(num_events=60_001)
    with tp.Context(0) as c:
        c.set_occupancy(precision, occ)
        c.set_events_per_thread(ept)
        gpu = c.run_batches(cfg, 0, cfg.num_batches, rng="xoshiro", precision=precision)
    ref = oracle.run_batches(cfg, 0, cfg.num_batches, tp.rng_flags("xoshiro"), tp.XOSHIRO_DEFAULT_SEED)
    if precision == tp.TP_PREC_FP64:
        assert_batches_close(gpu, ref)
    else:
        assert np.array_equal(gpu.selected, ref.selected)
        assert rel(gpu.sigma, ref.sigma) < 1e-6


@pytest.mark.parametrize("ept", [40, 41, 64, 100, 313, 333, 10000])
def test_events_per_thread_invariance(tp, oracle, cfg_valeurs, ept):
    cfg = cfg_valeurs.replace(num_events=30_000)
    with tp.Context(0) as c:
        c.set_events_per_thread(ept)
        gpu = c.run_batches(cfg, 0, 3, rng="xoshiro")
    ref = oracle.run_batches(cfg, 0, 3, tp.rng_flags("xoshiro"), tp.XOSHIRO_DEFAULT_SEED)
    assert_batches_close(gpu, ref)


def test_sqrts1000_configuration(tp, oracle, ctx, cfg_sqrts1000):
    cfg = cfg_sqrts1000
    nb = cfg.num_batches
    gpu = ctx.run_batches(cfg, 0, nb, rng="ranf")
    ref = oracle.run_batches(cfg, 0, nb, tp.rng_flags("ranf"), tp.RANF_DEFAULT_SEED)
    assert_batches_close(gpu, ref)
    a = tp.merge_finalize(cfg, gpu)
    b = tp.merge_finalize(cfg, ref)
    assert compare(a.res_data(), b.res_data(), rel_tol=1e-12) == []


def test_invalid_arguments(tp, ctx, cfg_valeurs):
    with pytest.raises(tp.TPError) as e:
        ctx.run_batches(cfg_valeurs.replace(num_events=0), 0, 1)
    assert e.value.code == tp.TP_ERR_INVALID
    with pytest.raises(tp.TPError) as e:
        ctx.run_batches(cfg_valeurs, 0, 1, rng="ranf", seed=2**40)
    assert e.value.code == tp.TP_ERR_INVALID
    with pytest.raises(tp.TPError) as e:
        ctx.set_events_per_thread(0)
    with pytest.raises(tp.TPError) as e:
        ctx.set_events_per_thread(39)  # 257 threads: beyond one CTA
    # batch ranges past the ABI's 2^46 limit, unknown precision and mode flags
    with pytest.raises(tp.TPError) as e:
        ctx.run_batches(cfg_valeurs, 2**46 + 1, 1, rng="xoshiro")
    assert e.value.code == tp.TP_ERR_INVALID
    with pytest.raises(tp.TPError) as e:
        ctx.run_batches(cfg_valeurs, 0, 1, rng="xoshiro", precision=7)
    assert e.value.code == tp.TP_ERR_INVALID
    acc = tp.BatchAccumulators(1)
    st = tp.library().tp_run_batches(ctx.h, ctypes.byref(cfg_valeurs.c), tp.TP_RNG_XOSHIRO256P | 0x800, 1, 0, 1,
                                     tp.TP_PREC_FP64, ctypes.byref(acc.soa()))
    assert st == tp.TP_ERR_INVALID
    # empty ranges are no-ops
    assert ctx.run_batches(cfg_valeurs, 0, 0, rng="xoshiro").n == 0
    # the context stays usable after errors
    ctx.run_batches(cfg_valeurs.replace(num_events=1000), 0, 1, rng="xoshiro")


@pytest.mark.parametrize("precision", [0, 1])
def test_ranf_reseed_outside_canonical_range(tp, oracle, ctx, cfg_valeurs, precision):
    """Batch 0's reseed 1000000970 leaves its state outside [0, 1e9)
    (tp_ranf_state_at refuses it): that batch's warps reach their events by
    stepping, the others by jump-ahead."""
    cfg = cfg_valeurs.replace(num_events=40_000)
    seed = 1000000970
    gpu = ctx.run_batches(cfg, 0, 4, rng="ranf", seed=seed, jump_per_batch=True, precision=precision)
    ref = oracle.run_batches(cfg, 0, 4, tp.rng_flags("ranf", True), seed)
    if precision == tp.TP_PREC_FP64:
        assert_batches_close(gpu, ref)
    else:
        assert np.array_equal(gpu.selected, ref.selected)
        assert rel(gpu.sigma, ref.sigma) < 1e-6


@pytest.mark.parametrize("rng", ["ranf", "xoshiro"])
@pytest.mark.parametrize("sincut", [0.2, 0.6])
def test_plane_cut(tp, oracle, ctx, cfg_valeurs, cfg_sqrts1000, rng, sincut):
    """The beam-plane cut (src/evcut.rs:77-92) is off in the shipped
    configurations (SINCUT = 0): here it is on, at both energies. FP64
    against the restatement; FP32-mixed must select the same events."""
    for base in (cfg_valeurs, cfg_sqrts1000):
        cfg = base.replace(num_events=80_000, beam_photon_plane_cut=sincut)
        nb = cfg.num_batches
        ref = oracle.run_batches(cfg, 0, nb, tp.rng_flags(rng), tp.default_seed(rng))
        unplaned = oracle.run_batches(base.replace(num_events=80_000), 0, nb, tp.rng_flags(rng), tp.default_seed(rng))
        assert ref.selected.sum() < unplaned.selected.sum()  # the cut removes events
        gpu = ctx.run_batches(cfg, 0, nb, rng=rng)
        assert_batches_close(gpu, ref)
        gpu32 = ctx.run_batches(cfg, 0, nb, rng=rng, precision=tp.TP_PREC_FP32_MIXED)
        assert np.array_equal(gpu32.selected, ref.selected)
        assert rel(gpu32.sigma, ref.sigma) < 1e-6


def test_plane_cut_dumps(tp, oracle, ctx, cfg_valeurs):
    """Event by event with the plane cut on: identical cut verdicts."""
    cfg = cfg_valeurs.replace(num_events=100_000, beam_photon_plane_cut=0.4)
    g = ctx.dump_events(cfg, 0, 20_000, rng="xoshiro")
    r = oracle.dump_events(cfg, tp.rng_flags("xoshiro"), tp.XOSHIRO_DEFAULT_SEED, 0, 20_000)
    assert np.array_equal(g["cut"], r["cut"])
    assert np.sum(r["cut"] == 4) > 0  # some events fail on the plane cut itself


def test_random_configurations(tp, oracle, ctx, cfg_sqrts1000):
    """Configurations drawn like the batched workload (sqrt(s) in [200, 2000],
    E_min in [1, 50], ACUT and BCUT in [0.80, 0.99], beta+- in [-1, 1]) plus
    a plane cut: FP64 per-batch sums against the restatement, FP32-mixed
    selecting the same events."""
    rng = np.random.default_rng(2024)
    for trial in range(6):
        cfg = cfg_sqrts1000.replace(
            num_events=30_000 + 1234 * trial, e_total=float(rng.uniform(200, 2000)), e_min=float(rng.uniform(1, 50)),
            beam_photons_cut=float(rng.uniform(0.8, 0.99)), photon_photon_cut=float(rng.uniform(0.8, 0.99)),
            beam_photon_plane_cut=float(rng.uniform(0.0, 0.3)), beta_plus=float(rng.uniform(-1, 1)),
            beta_minus=float(rng.uniform(-1, 1)))
        kind = "xoshiro" if trial % 2 else "ranf"
        nb = cfg.num_batches
        ref = oracle.run_batches(cfg, 0, nb, tp.rng_flags(kind), tp.default_seed(kind))
        assert_batches_close(ctx.run_batches(cfg, 0, nb, rng=kind), ref)
        gpu32 = ctx.run_batches(cfg, 0, nb, rng=kind, precision=tp.TP_PREC_FP32_MIXED)
        assert np.array_equal(gpu32.selected, ref.selected)
        assert rel(gpu32.sigma, ref.sigma) < 1e-6


@pytest.mark.parametrize("n", [1, 7, 10_001, 20_003])
@pytest.mark.parametrize("rng", ["ranf", "xoshiro"])
def test_tiny_and_ragged_runs(tp, oracle, ctx, cfg_valeurs, n, rng):
    """Runs of 1 and 7 events, and last batches of 1 and 3 events: most
    threads (and ranf warps) of those CTAs have no event."""
    cfg = cfg_valeurs.replace(num_events=n)
    nb = cfg.num_batches
    ref = oracle.run_batches(cfg, 0, nb, tp.rng_flags(rng), tp.default_seed(rng))
    assert_batches_close(ctx.run_batches(cfg, 0, nb, rng=rng), ref)
    gpu32 = ctx.run_batches(cfg, 0, nb, rng=rng, precision=tp.TP_PREC_FP32_MIXED)
    assert np.array_equal(gpu32.selected, ref.selected)
    fe = ctx.run_batches(cfg, 0, nb, rng=rng, faster_evgen=True)
    fe_ref = oracle.run_batches(cfg, 0, nb, tp.rng_flags(rng, faster_evgen=True), tp.default_seed(rng))
    assert_batches_close(fe, fe_ref)
