"""The FP64 logarithm of the event kernels (csrc/tp_math.h), on the CPU.

tp_log is built from IEEE basic operations only (FMA, multiply, add,
conversions) and one table, so the host build of the same header returns
the same bits as the device build. The reference's f64::ln is the C
library's log: these tests bound tp_log against it (at most 1 ulp apart,
equal in the great majority of cases) and against a 60-digit decimal
logarithm (faithfully rounded), and check that the committed table is the
one gen_log_table.py generates.
"""
import os
import struct
import subprocess
import sys
from decimal import Decimal, getcontext

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "3photons-rust_gb300", "csrc")

HARNESS = r"""
#include "tp_math.h"
#include <cstdio>
#include <cmath>
#include <vector>
int main(int argc, char** argv) {
  FILE* in = std::fopen(argv[1], "rb");
  std::vector<double> x;
  double v;
  while (std::fread(&v, 8, 1, in) == 1) x.push_back(v);
  std::fclose(in);
  FILE* out = std::fopen(argv[2], "wb");
  for (double a : x) {
    const double r[2] = {tp::tp_log(a), std::log(a)};
    std::fwrite(r, 8, 2, out);
  }
  std::fclose(out);
  return 0;
}
"""


@pytest.fixture(scope="module")
def tp_log_cpu(tmp_path_factory):
    d = tmp_path_factory.mktemp("tp_log")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    exe = d / "h"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)],
                   check=True)

    def run(x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        fin, fout = d / "in.bin", d / "out.bin"
        x.tofile(fin)
        subprocess.run([str(exe), str(fin), str(fout)], check=True)
        r = np.fromfile(fout, dtype=np.float64).reshape(-1, 2)
        return r[:, 0], r[:, 1]

    return run


def ulp_diff(a, b):
    ia = a.view(np.int64)
    ib = b.view(np.int64)
    return np.abs(ia - ib)


def test_log_table_is_generated(tmp_path):
    out = subprocess.run([sys.executable, os.path.join(CSRC, "gen_log_table.py")], check=True,
                         capture_output=True, text=True).stdout
    with open(os.path.join(CSRC, "tp_log_table.h")) as fh:
        assert fh.read() == out


def test_log_matches_libm_on_event_arguments(tp_log_cpu):
    """The kernels take log of em = r1 r2 (two draws in [0, 1)), or of the
    smallest normal double when that product is 0."""
    rng = np.random.default_rng(20240611)
    n = 1_000_000
    u = (rng.integers(0, 2**53, size=(2, n), dtype=np.int64).astype(np.float64)) * 2.0**-53
    em = u[0] * u[1]
    em[em == 0.0] = np.finfo(np.float64).tiny
    a, b = tp_log_cpu(em)
    d = ulp_diff(a, b)
    assert d.max() <= 1
    assert (d == 0).mean() > 0.99


def test_log_matches_libm_across_ranges(tp_log_cpu):
    rng = np.random.default_rng(7)
    n = 400_000
    parts = [
        rng.random(n),                                          # [0, 1)
        1.0 + (rng.random(n) - 0.5) * 0.05,                     # around 1, both branches
        1.0 + (rng.random(n) - 0.5) * 2.0**-20,                 # very close to 1
        np.ldexp(1.0 + rng.random(n), rng.integers(-1022, 1023, n)),  # every exponent
    ]
    x = np.concatenate(parts)
    x = x[x > 0]
    a, b = tp_log_cpu(x)
    d = ulp_diff(a, b)
    assert d.max() <= 1
    assert (d == 0).mean() > 0.99


def test_log_special_arguments(tp_log_cpu):
    tiny = np.finfo(np.float64).tiny
    x = np.array([1.0, 2.0, 0.5, 0.25, 1.0 - 2.0**-53, 1.0 + 2.0**-52, 1.0 - 1.0 / 64, 1.0 + 1.0 / 64,
                  tiny, np.nextafter(1.0, 0.0), 1.7976931348623157e308, 5e-324, 0.0, -1.0, np.inf, np.nan])
    a, b = tp_log_cpu(x)
    assert a[0] == 0.0 and not np.signbit(a[0])
    assert ulp_diff(a[:12], b[:12]).max() <= 1
    # arguments outside the positive normal range take the C library's path
    assert a[12] == -np.inf and np.isnan(a[13]) and a[14] == np.inf and np.isnan(a[15])
    assert a[11] == b[11]


def test_log_faithful_against_decimal(tp_log_cpu):
    getcontext().prec = 60
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.random(1500) * rng.random(1500), 1.0 + (rng.random(500) - 0.5) * 0.05])
    x = x[x > 0]
    a, _ = tp_log_cpu(x)
    for xi, ai in zip(x, a):
        exact = Decimal(float(xi)).ln()
        lo, hi = np.nextafter(ai, -np.inf), np.nextafter(ai, np.inf)
        # the exact value lies strictly between the neighbours of the result
        assert Decimal(float(lo)) < exact < Decimal(float(hi)), (xi, ai)
