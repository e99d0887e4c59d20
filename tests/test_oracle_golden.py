"""Pins the CPU restatement (the checker) to the reference's own goldens:
every feature set the reference's CI compares (ci.yml:130-203) at its
`valeurs` input, N = 1e7. Byte-exact where the reference's run is
deterministic; the xoshiro + faster-threading golden was merged in thread
completion order, for which the reference's CI allows -a 1.1e-16."""
import os
import subprocess

import pytest

from conftest import GOLDEN, golden
from numdiff import compare

MODES = [
    ("", []),
    ("multi-threading", []),
    ("no-photon-sorting", ["--no-photon-sorting"]),
    ("standard-random", ["--rng", "xoshiro"]),
    ("standard-random,multi-threading", ["--rng", "xoshiro"]),
    ("multi-threading,faster-threading", ["--jump-per-batch"]),
    ("standard-random,multi-threading,faster-threading", ["--rng", "xoshiro", "--jump-per-batch"]),
    ("faster-evgen", ["--faster-evgen"]),
]


@pytest.mark.parametrize("features,args", MODES, ids=[m[0] or "default" for m in MODES])
def test_oracle_reproduces_golden(oracle, tmp_path, features, args):
    import tp_oracle_py

    threads = "1" if "faster-evgen" in features else str(os.cpu_count() or 1)
    out = subprocess.run([tp_oracle_py.CLI, "-c", os.path.join(GOLDEN, "valeurs"), "-o", str(tmp_path / "res.data"),
                          "--threads", threads, *args], check=True, capture_output=True, text=True).stdout
    res = (tmp_path / "res.data").read_text()
    assert out == golden("stdout.log", features)
    if features == "standard-random,multi-threading,faster-threading":
        assert compare(res, golden("res.data", features), abs_tol=1.1e-16) == []
    else:
        assert res == golden("res.data", features)
