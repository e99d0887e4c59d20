"""Checkpoint / resume at batch granularity: a run interrupted after some
chunks (the failure is injected on the host) and restarted from its
checkpoint equals the uninterrupted run bit for bit. The batch runner is the
CPU restatement here; on a GPU it is Context.run_batches."""
import pytest


class Crash(RuntimeError):
    pass


@pytest.mark.parametrize("rng,jump", [("ranf", False), ("xoshiro", True)])
def test_resume_after_injected_failure(tp, oracle, cfg_valeurs, tmp_path, rng, jump):
    cfg = cfg_valeurs.replace(num_events=93_456)  # 10 batches, the last partial
    kind = tp.rng_flags(rng, jump)
    seed = tp.default_seed(rng)
    calls = []

    def runner(first, n, fail_at=None):
        calls.append(first)
        if fail_at is not None and first >= fail_at:
            raise Crash("injected failure at batch %d" % first)
        return oracle.run_batches(cfg, first, n, kind, seed, threads=1)

    ckpt = str(tmp_path / "run.npz")
    with pytest.raises(Crash):
        tp.run_simulation_resumable(cfg, ckpt, lambda f, n: runner(f, n, fail_at=6), chunk_batches=3)
    assert calls == [0, 3, 6]
    res = tp.run_simulation_resumable(cfg, ckpt, runner, chunk_batches=3)
    assert calls[3:] == [6, 9]  # resumed at the first missing batch
    whole = oracle.run_batches(cfg, 0, cfg.num_batches, kind, seed)
    assert bytes(res.c) == bytes(tp.merge_finalize(cfg, whole).c)


def test_checkpoint_of_another_run_is_refused(tp, oracle, cfg_valeurs, tmp_path):
    ckpt = str(tmp_path / "run.npz")
    cfg = cfg_valeurs.replace(num_events=20_000)
    run = lambda f, n: oracle.run_batches(cfg, f, n, 0, tp.RANF_DEFAULT_SEED, threads=1)
    tp.run_simulation_resumable(cfg, ckpt, run, chunk_batches=1)
    with pytest.raises(ValueError):
        tp.run_simulation_resumable(cfg.replace(num_events=30_000), ckpt, run)


def test_checkpoint_keyed_on_configuration_and_run(tp, oracle, cfg_valeurs, tmp_path):
    """Same event count, other physics or other stream: refused."""
    ckpt = str(tmp_path / "run.npz")
    cfg = cfg_valeurs.replace(num_events=20_000)
    run = lambda f, n: oracle.run_batches(cfg, f, n, 0, tp.RANF_DEFAULT_SEED, threads=1)
    tp.run_simulation_resumable(cfg, ckpt, run, chunk_batches=1, run_key="ranf 234612947")
    with pytest.raises(ValueError):
        tp.run_simulation_resumable(cfg.replace(beta_plus=0.5), ckpt, run, run_key="ranf 234612947")
    with pytest.raises(ValueError):
        tp.run_simulation_resumable(cfg, ckpt, run, run_key="ranf 1")
    # the same run resumes (nothing left to do)
    res = tp.run_simulation_resumable(cfg, ckpt, run, run_key="ranf 234612947")
    assert res.selected_events > 0
