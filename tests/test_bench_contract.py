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
    for f in (t["source"].split(":")[0], i["source"].split(":")[0]):
        assert os.path.exists(os.path.join(ROOT, f)), f
