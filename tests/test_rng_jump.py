"""Jump-ahead of both random streams (host side of the library) against the
CPU restatement's stepping: ranf (src/random/ranf.rs) and xoshiro256+
(src/random/standard.rs), including the 2^128 RandomGenerator::jump, which
the restatement computes by squaring the generator's 256x256 GF(2) matrix
and the library by Berlekamp-Massey + polynomial powers."""
import ctypes

import numpy as np
import pytest


def xo_state_at(tp, seed, jumps, draws):
    s = (ctypes.c_uint64 * 4)()
    assert tp.library().tp_xoshiro_state_at(seed, jumps, draws, s) == 0
    return list(s)


def xo_next(s):
    m = (1 << 64) - 1
    r = (s[0] + s[3]) & m
    t = (s[1] << 17) & m
    s[2] ^= s[0]
    s[3] ^= s[1]
    s[1] ^= s[2]
    s[0] ^= s[3]
    s[2] ^= t
    s[3] = ((s[3] << 45) | (s[3] >> 19)) & m
    return r


@pytest.mark.parametrize("seed", [12345, 0, 2**63 + 7])
@pytest.mark.parametrize("draws", [0, 1, 11, 12, 255, 256, 257, 120000, 1234567])
def test_xoshiro_jump_equals_stepping(tp, oracle, seed, draws):
    got = xo_state_at(tp, seed, 0, draws)
    ref = oracle.xoshiro_state(seed, 0)
    if draws <= 1234567:
        for _ in range(draws):
            xo_next(ref)
    assert got == ref
    # the uniforms the stream yields from there match the restatement's
    u = oracle.draws(tp.TP_RNG_XOSHIRO256P, seed, 0, draws, 4)
    s = list(got)
    mine = [(xo_next(s) >> 11) * 2.0**-53 for _ in range(4)]
    assert mine == u.tolist()


@pytest.mark.parametrize("jumps", [1, 2, 3, 17])
def test_xoshiro_jump128_matches_matrix_method(tp, oracle, jumps):
    assert xo_state_at(tp, 12345, jumps, 0) == oracle.xoshiro_state(12345, jumps)


def test_xoshiro_jump_then_draws(tp, oracle):
    got = xo_state_at(tp, 12345, 5, 1000)
    ref = oracle.xoshiro_state(12345, 5)
    for _ in range(1000):
        xo_next(ref)
    assert got == ref


@pytest.mark.parametrize("draws", [0, 1, 54, 55, 56, 109, 110, 120000, 3 * 120000 + 17, 10**7 + 3])
def test_ranf_jump_equals_stepping(tp, oracle, draws):
    slots = (ctypes.c_int32 * 55)()
    index = ctypes.c_int32()
    assert tp.library().tp_ranf_state_at(234612947, draws, slots, ctypes.byref(index)) == 0
    # reference: the state after r resets beyond the warm-up, index 55 - m
    r, m = divmod(draws, 55)
    ref = oracle.ranf_state(234612947, r)
    assert list(slots) == ref[:55]
    assert index.value == 55 - m
    # the next draws agree with the restatement's stream
    nxt = oracle.draws(tp.TP_RNG_RANF, 234612947, 0, draws, 3)
    idx = index.value
    vals = list(slots)
    mine = []
    for _ in range(3):
        if idx == 0:
            ref2 = oracle.ranf_state(234612947, r + 1)
            vals = ref2[:55]
            idx = 55
        idx -= 1
        mine.append(vals[idx] * 1e-9)
    assert mine == nxt.tolist()


def test_ranf_noncanonical_seed_rejected(tp, oracle):
    slots = (ctypes.c_int32 * 55)()
    index = ctypes.c_int32()
    # seeds beyond 1e9 (reached by the per-batch reseeding after ~6200
    # batches) leave the state outside [0, 1e9): no linear jump-ahead
    assert tp.library().tp_ranf_state_at(1_000_000_970, 100, slots, ctypes.byref(index)) == tp.TP_ERR_UNSUPPORTED
    st = oracle.ranf_state(1_000_000_970, 0)[:55]
    assert any(v < 0 or v >= 10**9 for v in st)


def test_jumped_stream_is_per_batch_stream(tp, oracle, cfg_valeurs):
    """The restatement's stream of scan point p (seed jumped p times) starts
    where batch p of the per-batch-jump mode starts, for both generators."""
    cfg = cfg_valeurs.replace(num_events=60_000)
    for rng in ("xoshiro", "ranf"):
        kind, seed = tp.rng_flags(rng), tp.default_seed(rng)
        for p in (1, 4):
            a = oracle.run_batches_jumped(cfg, 0, 1, kind, seed, p, threads=1).as_array()
            b = oracle.run_batches(cfg, p, 1, tp.rng_flags(rng, jump_per_batch=True), seed, threads=1).as_array()
            assert np.array_equal(a, b), (rng, p)
