"""bench.py's contract on the CPU: the reference arm (the CPU restatement on
the host cores; no GPU needed) prints one JSON line with the keys the
benchmark line must carry, and the per-kernel figures bench.py reads from
profiles/ are present and well-formed."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line(oracle):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "events/s"
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]


def test_profile_figures():
    t = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    assert t["kernel"] == "k_events_xoshiro_fp64" and 0 < t["bytes_per_event"] < 1
    i = json.load(open(os.path.join(ROOT, "profiles", "issue.json")))
    assert i["kernel"] == "k_events_xoshiro_fp32" and 10 < i["warp_inst_per_event"] < 100
    # per kernel variant (CTAs per SM), as the bench looks them up
    assert set(i["by_variant"]) <= {"2", "3", "4"} and all(10 < v < 100 for v in i["by_variant"].values())
    for f in (t["source"].split(":")[0], i["source"].split(":")[0]):
        assert os.path.exists(os.path.join(ROOT, f)), f


def test_compact_line():
    """The printed line stays short (a few KB: a driver keeps the tail of the
    output) and ends with the precision form's headline figures."""
    sys.path.insert(0, ROOT)
    import bench

    fp32 = {"value": 3.4e10, "kernel": "k_events_xoshiro_fp32", "kernel_ms": 290.1, "autotuned_events_per_thread": 157,
            "kernel_variant_ctas_per_sm": 4, "rechecked_fraction": 1.6e-4, "ratio_vs_fp64": 35.8,
            "roofline": {"frac": 0.31, "sfu_frac": 0.18, "issue": {"frac": 0.85}},
            "e2e": {"value": 3.39e10, "unit": "events/s", "h2d_bytes_per_step": 136, "d2h_bytes_per_step": 104000000},
            "accuracy_vs_fp64": {"selected_equal": True, "max_rel_err": 1.6e-7,
                                 "rel_err": {"sigma": 4.3e-8, "beta_min": 2.2e-8, "spm2_1_A": 2.8e-8,
                                             "spm2_1_B+": 1.7e-8, "ss_p": 3e-8}}}
    grad = {"forward_ms": 38.1, "adjoint_ms": 33.9, "grad_over_fwd": 0.89,
            "at_test_point": {"theta": [0.25, -0.1, 91.187, 2.49], "dlnL_dtheta": [1.0, 2.0, 3.0, 4.0],
                              "max_rel_dev_vs_analytic": 1e-10, "max_rel_dev_vs_central_diff": 1e-9},
            "flipped_bins": 0, "fit": {"beta": [0.3, -0.2], "beta_err": [7e-5, 6e-5]}}
    d = {"metric": bench.METRIC, "value": 9.48e8, "unit": "events/s", "n_gpus": 1, "steps": 20, "warmup": 5,
         "ms_per_step": 1054.6, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
         "data": "synthetic", "gpu_launches": 80,
         "config": {"l2": "flushed between steps (256 MiB write)", "parallelism": "batch-range shards",
                    "autotuned_events_per_thread": 313, "kernel_variant_ctas_per_sm": 2},
         "roofline": {"bound": "fp64", "achieved": 1.185, "peak": 1.054, "unit": "TFLOP/s", "frac": 1.12,
                      "traffic": 3.2e7, "kernel": "k_events_xoshiro_fp64", "frac_fixed": {"frac": 0.95},
                      "fp64_pipe_active_ncu": 0.862},
         "cpu_baseline": {"value": 2.36e7, "unit": "events/s", "cores": 16, "kind": "port", "value_1core": 4.5e6,
                          "sample": "first 5927 batches"},
         "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 105},
         "e2e": {"value": 9.47e8, "unit": "events/s", "h2d_bytes_per_step": 136, "d2h_bytes_per_step": 10400000},
         "fp32_mixed": fp32, "grad": grad,
         "batched": {"value": 3.08e10, "e2e": 2.9e10, "events_per_step": 5578252194, "points": 256},
         "ranf": {"fp64": 9.26e8, "fp32": 2.25e10, "fp32_over_xoshiro": 0.66},
         "faster_evgen": [{"rng": "xoshiro", "events_per_s": 7.9e8, "boundary_pass_ms": 234.0, "ms_per_step": 1262.0},
                          {"rng": "ranf", "events_per_s": 6.2e8, "boundary_pass_ms": 92.0, "ms_per_step": 322.0}]}
    line = json.dumps(bench.compact_line(d, "gpurun_out/bench_detail.json"))
    assert len(line) < 2600, len(line)
    out = json.loads(line)
    assert list(out)[-5:] == ["fp32_mixed_value", "fp32_mixed_e2e", "fp32_over_fp64", "fp32_max_rel_err",
                              "grad_over_fwd"]
    assert out["value"] == 9.48e8 and out["fp32_over_fp64"] == 35.8 and out["roofline"]["frac_fixed"] == 0.95
    tail = line[-400:]
    assert '"fp32_mixed_value": 34000000000.0' in tail and '"grad_over_fwd": 0.89' in tail
