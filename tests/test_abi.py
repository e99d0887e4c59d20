"""The C ABI library loads without a GPU and exports every function that
include/*.h declares; struct layouts agree between C and the ctypes mirror;
GPU entry points fail cleanly (no abort) when no device is usable."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include"))) if f.endswith(".h")]


def declared_functions():
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(tp_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_headers_declare_functions():
    names = declared_functions()
    assert "tp_run_batches" in names and "tp_create" in names and len(names) >= 15


@pytest.mark.parametrize("name", declared_functions())
def test_symbol_exported(tp, name):
    assert hasattr(tp.library(), name), name


def test_struct_layouts(tp, tmp_path):
    src = tmp_path / "layout.c"
    src.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "tp_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(tp_config), sizeof(tp_batch_soa), sizeof(tp_event_dump),
         sizeof(tp_final_results), offsetof(tp_config, num_bins), offsetof(tp_event_dump, cut),
         offsetof(tp_final_results, sigma));
  return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [ctypes.sizeof(tp.CConfig), ctypes.sizeof(tp.CBatchSoa), ctypes.sizeof(tp.CEventDump),
            ctypes.sizeof(tp.CFinalResults), tp.CConfig.num_bins.offset, tp.CEventDump.cut.offset,
            tp.CFinalResults.sigma.offset]
    assert got == want


def test_create_fails_cleanly_without_device(tp):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(tp.TPError) as e:
        tp.Context(0)
    assert e.value.code == tp.TP_ERR_NO_DEVICE


def test_null_context_rejected(tp):
    lib = tp.library()
    cfg = tp.CConfig()
    soa = tp.CBatchSoa()
    assert lib.tp_run_batches(None, ctypes.byref(cfg), 0, 0, 0, 1, 0, ctypes.byref(soa)) == tp.TP_ERR_INVALID
    assert lib.tp_dump_events(None, ctypes.byref(cfg), 0, 0, 0, 1, None) == tp.TP_ERR_INVALID
    assert lib.tp_get_tuning(None, 0, None, None) == tp.TP_ERR_INVALID
    assert lib.tp_set_fe_store_cap(None, 0) == tp.TP_ERR_INVALID
    assert lib.tp_grad(None, ctypes.byref(cfg), 0, 0, 0, 1, 0, None, None, None, None) == tp.TP_ERR_INVALID
