"""tp_run_batches_noalloc, the entry point for callers that cannot allocate
GPU memory (memory planned once at start-up, a foreign allocator that owns
the GPU's memory): called through the C ABI on the current device with
output arrays the test owns, twice in a row, against the regular entry
point tp_run_batches on the same batches. The library's fixed working memory is
shared by both calls; the second call must not see the first one's data.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process (the
first call sets the device up)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def device_outputs(torch, n):
    sel = torch.zeros(n, dtype=torch.int64, device="cuda")
    f = torch.zeros(12 * n, dtype=torch.float64, device="cuda")
    return sel, f


def call_noalloc(tp, torch, cfg, first, n, precision, flags=0):
    sel, f = device_outputs(torch, n)
    base = f.data_ptr()
    soa = tp.CBatchSoa(ctypes.c_void_p(sel.data_ptr()), ctypes.c_void_p(base), ctypes.c_void_p(base + 5 * n * 8),
                       ctypes.c_void_p(base + 10 * n * 8), ctypes.c_void_p(base + 11 * n * 8))
    stream = torch.cuda.current_stream().cuda_stream
    st = tp.library().tp_run_batches_noalloc(ctypes.byref(cfg.c), tp.TP_RNG_XOSHIRO256P | flags,
                                             tp.XOSHIRO_DEFAULT_SEED, first, n, precision, ctypes.byref(soa),
                                             ctypes.c_void_p(stream))
    assert st == 0, tp.library().tp_last_error(None)
    torch.cuda.synchronize()
    acc = tp.BatchAccumulators(n)
    acc.selected[:] = sel.cpu().numpy().astype(np.uint64)
    fa = f.cpu().numpy()
    acc.spm2[:] = fa[:5 * n].reshape(5, n)
    acc.vars[:] = fa[5 * n:10 * n].reshape(5, n)
    acc.sigma[:] = fa[10 * n:11 * n]
    acc.variance[:] = fa[11 * n:]
    return acc


def assert_same(a, b):
    # the tolerance of the other batch tests: counts exact, sums 1e-12
    assert np.array_equal(a.selected, b.selected)
    for name in ("spm2", "vars", "sigma", "variance"):
        x, y = getattr(a, name), getattr(b, name)
        assert np.all(np.abs(x - y) <= 1e-12 * np.maximum(np.abs(y), 1e-300)), name


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32-mixed"])
def test_noalloc_matches_regular_entry_point_twice(tp, cfg_valeurs, precision):
    torch = pytest.importorskip("torch")
    cfg = cfg_valeurs.replace(num_events=3_000_000)
    with tp.Context(0) as ctx:
        ref_a = ctx.run_batches(cfg, 17, 40, rng="xoshiro", precision=precision)
        ref_b = ctx.run_batches(cfg, 250, 9, rng="xoshiro", precision=precision, jump_per_batch=True)
    # two calls in a row on different batches: the second must not be
    # affected by what the first left in the shared working memory
    first = call_noalloc(tp, torch, cfg, 17, 40, precision)
    second = call_noalloc(tp, torch, cfg, 250, 9, precision, tp.TP_MODE_JUMP_PER_BATCH)
    assert_same(first, ref_a)
    assert_same(second, ref_b)
    again = call_noalloc(tp, torch, cfg, 17, 40, precision)
    assert_same(again, ref_a)
    # the other accepted flag: photons left in generation order
    with tp.Context(0) as ctx:
        ref_c = ctx.run_batches(cfg, 3, 5, rng="xoshiro", precision=precision, sorting=False)
    unsorted = call_noalloc(tp, torch, cfg, 3, 5, precision, tp.TP_MODE_NO_PHOTON_SORTING)
    assert_same(unsorted, ref_c)


def test_noalloc_rejects_oversized_ranges(tp, cfg_valeurs):
    torch = pytest.importorskip("torch")
    sel, f = device_outputs(torch, 1)
    soa = tp.CBatchSoa(*[ctypes.c_void_p(p) for p in (sel.data_ptr(), f.data_ptr(), f.data_ptr(), f.data_ptr(),
                                                        f.data_ptr())])
    lib = tp.library()
    st = lib.tp_run_batches_noalloc(ctypes.byref(cfg_valeurs.c), tp.TP_RNG_XOSHIRO256P, 1, 0, 4097, 0,
                                    ctypes.byref(soa), None)
    assert st == tp.TP_ERR_INVALID
    assert b"TP_NOALLOC_MAX_BATCHES" in lib.tp_last_error(None)
    st = lib.tp_run_batches_noalloc(ctypes.byref(cfg_valeurs.c), tp.TP_RNG_RANF, 1, 0, 1, 0, ctypes.byref(soa), None)
    assert st == tp.TP_ERR_INVALID
