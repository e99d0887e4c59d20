"""The host side kept from the reference: valeurs parsing and echo
(src/config.rs), ordered merge + finalize (src/resacc.rs:133-223) and the
writers (src/output.rs, src/resfin.rs), checked against the goldens and the
CPU restatement."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden


def test_config_load_matches_restatement(tp, oracle, valeurs):
    cfg = tp.Configuration.load(valeurs, echo=False)
    st, ref, echo = oracle.load(valeurs)
    assert st == 0
    assert cfg.as_dict() == ref.as_dict()
    buf = ctypes.create_string_buffer(4096)
    c = tp.CConfig()
    assert tp.library().tp_config_load(valeurs.encode(), ctypes.byref(c), buf, 4096) == 0
    assert buf.value.decode() == echo
    # the echo is the first 18 lines of the reference's stdout
    assert golden("stdout.log", "").startswith(echo)


@pytest.mark.parametrize("line,value", [(0, "0"), (16, ".true."), (17, ".TRUE."), (1, "abc"), (0, "-5")])
def test_config_checks(tp, tmp_path, valeurs, line, value):
    lines = open(valeurs).read().splitlines()
    parts = lines[line].split(None, 1)
    lines[line] = value + ("\t" + parts[1] if len(parts) > 1 else "")
    p = tmp_path / "valeurs"
    p.write_text("\n".join(lines) + "\n")
    with pytest.raises(tp.TPError) as e:
        tp.Configuration.load(str(p), echo=False)
    assert e.value.code == tp.TP_ERR_INVALID


def test_config_missing_items(tp, tmp_path):
    p = tmp_path / "valeurs"
    p.write_text("10\n91.187\n")
    with pytest.raises(tp.TPError):
        tp.Configuration.load(str(p), echo=False)
    with pytest.raises(tp.TPError) as e:
        tp.Configuration.load(str(tmp_path / "nope"), echo=False)
    assert e.value.code == tp.TP_ERR_IO


@pytest.fixture(scope="module")
def golden_batches(oracle, cfg_valeurs, tp):
    return oracle.run_batches(cfg_valeurs, 0, cfg_valeurs.num_batches, tp.TP_RNG_RANF, tp.RANF_DEFAULT_SEED)


def test_merge_finalize_and_writers_match_golden(tp, oracle, cfg_valeurs, golden_batches, tmp_path):
    res = tp.merge_finalize(cfg_valeurs, golden_batches)
    assert res.res_data() == golden("res.data", "")
    gold = golden("stdout.log", "")
    assert gold.endswith(res.report())
    # the restatement's finalize gives the same bits
    ref = oracle.merge_finalize(cfg_valeurs, golden_batches)
    assert bytes(ref) == bytes(res.c)
    # file writers
    tp.dump_results(cfg_valeurs, res, 1.25, str(tmp_path), timestamp="03-Dec-26 12:00:00")
    assert (tmp_path / "res.data").read_text() == golden("res.data", "")
    times = (tmp_path / "res.times").read_text().splitlines()
    assert times[0] == " 03-Dec-26 12:00:00"
    assert times[2] == " Temps ecoule                   : ???"
    assert times[3] == " Temps ecoule utilisateur       : 1.25"
    assert times[5] == " Temps ecoule par evenement     : 1.2500000000000e-7"
    pil = (tmp_path / "pil.mc").read_text().splitlines()
    assert pil[0] == "03-Dec-26 12:00:00"
    vals = [float(x) for x in pil[1].split()]
    assert vals[0] == 91.187 and vals[-1] == res.sigma
    tp.dump_results(cfg_valeurs, res, 1.25, str(tmp_path), timestamp="03-Dec-26 12:00:01")
    assert len((tmp_path / "pil.mc").read_text().splitlines()) == 4  # appended


def test_merge_is_in_batch_order(tp, cfg_valeurs, golden_batches):
    # merging is ResultsAccumulator::merge left to right: a permuted order
    # may change the last bits, the original order reproduces them exactly
    a = tp.merge_finalize(cfg_valeurs, golden_batches)
    b = tp.merge_finalize(cfg_valeurs, golden_batches)
    assert bytes(a.c) == bytes(b.c)


def test_event_weight(tp, oracle):
    w = ctypes.c_double()
    for e in (91.187, 1000.0, 200.0, 2000.0):
        assert tp.library().tp_event_weight(e, ctypes.byref(w)) == 0
        assert w.value == oracle.L.tpo_event_weight(e)
