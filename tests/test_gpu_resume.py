"""Checkpoint / resume with the GPU as the batch runner: a run interrupted
after some chunks (failure injected on the host, between launches) and
restarted from its checkpoint equals the uninterrupted GPU run bit for bit,
for the default and the faster-evgen generation."""
import pytest

pytestmark = pytest.mark.gpu


class Crash(RuntimeError):
    pass


@pytest.mark.parametrize("rng,fe", [("xoshiro", False), ("ranf", False), ("ranf", True)])
def test_gpu_resume_after_injected_failure(tp, ctx, cfg_valeurs, tmp_path, rng, fe):
    cfg = cfg_valeurs.replace(num_events=231_234)  # 24 batches, the last partial
    key = "%s %s fe=%d" % (rng, tp.default_seed(rng), fe)

    def runner(first, n, fail_at=None):
        if fail_at is not None and first >= fail_at:
            raise Crash("injected failure at batch %d" % first)
        return ctx.run_batches(cfg, first, n, rng=rng, faster_evgen=fe)

    ckpt = str(tmp_path / "run.npz")
    with pytest.raises(Crash):
        tp.run_simulation_resumable(cfg, ckpt, lambda f, n: runner(f, n, fail_at=10), chunk_batches=5, run_key=key)
    res = tp.run_simulation_resumable(cfg, ckpt, runner, chunk_batches=5, run_key=key)
    whole = tp.run_simulation(cfg, rng=rng, faster_evgen=fe, ctx=ctx)
    assert bytes(res.c) == bytes(whole.c)
