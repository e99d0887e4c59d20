"""`tp_run`, the command-line program (the reference's main(), src/main.rs:
75-145, on the GPU): stdout and res.data against the reference's goldens,
res.times and pil.mc written."""
import os
import subprocess

import pytest

from conftest import GOLDEN, ROOT, golden
from numdiff import compare

pytestmark = pytest.mark.gpu

CLI = os.path.join(ROOT, "3photons-rust_gb300", "tp_run")


def differing_fields(a, b):
    """Whitespace-separated fields whose printed text differs."""
    ta, tb = a.split(), b.split()
    return sum(x != y for x, y in zip(ta, tb)) + abs(len(ta) - len(tb))


@pytest.mark.parametrize("features,args", [("", []), ("standard-random", ["--rng", "xoshiro"]),
                                           ("multi-threading,faster-threading", ["--jump-per-batch"]),
                                           ("faster-evgen", ["--faster-evgen"])])
def test_tp_run_reproduces_golden(tmp_path, record_property, features, args):
    out = subprocess.run([CLI, "-c", os.path.join(GOLDEN, "valeurs"), "-d", str(tmp_path), *args],
                         capture_output=True, text=True, check=True).stdout
    assert compare(out, golden("stdout.log", features), rel_tol=1e-12) == []
    res = (tmp_path / "res.data").read_text()
    assert res.splitlines()[1] == golden("res.data", features).splitlines()[1]
    assert compare(res, golden("res.data", features), rel_tol=1e-12) == []
    # beyond the numeric comparison: the printed fields (14 and 8
    # significant digits) equal the golden's text byte for byte
    n_res, n_out = differing_fields(res, golden("res.data", features)), differing_fields(out, golden("stdout.log",
                                                                                                     features))
    record_property("res_data_fields_differing", n_res)
    record_property("stdout_fields_differing", n_out)
    assert n_res == 0 and n_out == 0, (n_res, n_out)
    assert (tmp_path / "res.times").read_text().count("\n") == 6
    assert len((tmp_path / "pil.mc").read_text().splitlines()) == 2


def test_tp_run_rejects_bad_config(tmp_path):
    bad = tmp_path / "valeurs"
    text = open(os.path.join(GOLDEN, "valeurs")).read().splitlines()
    text[17] = ".true.\t'HBookage'"
    bad.write_text("\n".join(text) + "\n")
    p = subprocess.run([CLI, "-c", str(bad), "-d", str(tmp_path)], capture_output=True, text=True)
    assert p.returncode == 1 and "configuration" in p.stderr
