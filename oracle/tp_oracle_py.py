"""ctypes wrapper of the CPU restatement (libtp_oracle.so).

Test infrastructure only: used by tests/, by __graft_entry__.smoke() as the
checker, and by bench.py's CPU-baseline leg. The product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libtp_oracle.so")
CLI = os.path.join(HERE, "tp_oracle")
TPO_MODE_FASTER_EVGEN = 0x400


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib(pkg):
    """Loads the oracle; `pkg` is the product's Python package, whose ctypes
    struct definitions mirror the shared ABI header."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        u64, i32, vp = ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p
        L.tpo_config_load.argtypes = [ctypes.c_char_p, P(pkg.CConfig), ctypes.c_char_p, ctypes.c_size_t]
        L.tpo_event_weight.restype = ctypes.c_double
        L.tpo_event_weight.argtypes = [ctypes.c_double]
        L.tpo_couplings.argtypes = [P(pkg.CConfig), P(ctypes.c_double)]
        L.tpo_sigma_contribs.argtypes = [P(pkg.CConfig), P(ctypes.c_double)]
        L.tpo_draws.argtypes = [i32, u64, u64, u64, u64, P(ctypes.c_double)]
        L.tpo_xoshiro_state.argtypes = [u64, u64, P(ctypes.c_uint64)]
        L.tpo_xoshiro_jump128.argtypes = [P(ctypes.c_uint64)]
        L.tpo_ranf_state.argtypes = [ctypes.c_int32, u64, P(ctypes.c_int32)]
        L.tpo_dump_events.argtypes = [P(pkg.CConfig), i32, u64, u64, u64, vp]
        L.tpo_m2_sums_of.argtypes = [P(pkg.CConfig), P(ctypes.c_double), P(ctypes.c_double)]
        L.tpo_run_batches.argtypes = [P(pkg.CConfig), i32, u64, u64, u64, P(pkg.CBatchSoa), i32]
        L.tpo_run_batches_jumped.argtypes = [P(pkg.CConfig), i32, u64, u64, u64, u64, P(pkg.CBatchSoa), i32]
        d = ctypes.c_double
        L.tpo_binned.argtypes = [P(pkg.CConfig), i32, u64, u64, u64, i32, i32, d, d, d, d, vp]
        L.tpo_merge_finalize.argtypes = [P(pkg.CConfig), P(pkg.CBatchSoa), u64, P(pkg.CFinalResults)]
        L.tpo_format_res_data.argtypes = [P(pkg.CConfig), P(pkg.CFinalResults), ctypes.c_char_p, ctypes.c_size_t]
        L.tpo_format_report.argtypes = [P(pkg.CConfig), P(pkg.CFinalResults), ctypes.c_char_p, ctypes.c_size_t]
        _lib = L
    return _lib


class Oracle:
    def __init__(self, pkg):
        self.pkg = pkg
        self.L = lib(pkg)

    def load(self, path):
        c = self.pkg.CConfig()
        buf = ctypes.create_string_buffer(4096)
        st = self.L.tpo_config_load(path.encode(), ctypes.byref(c), buf, len(buf))
        return st, self.pkg.Configuration(c), buf.value.decode()

    def run_batches(self, cfg, first_batch, n_batches, rng_kind, seed, threads=None):
        acc = self.pkg.BatchAccumulators(n_batches)
        soa = acc.soa()
        threads = threads or os.cpu_count() or 1
        st = self.L.tpo_run_batches(ctypes.byref(cfg.c), rng_kind, seed, first_batch, n_batches,
                                    ctypes.byref(soa), threads)
        assert st == 0, st
        return acc

    def run_batches_jumped(self, cfg, first_batch, n_batches, rng_kind, seed, jumps, threads=None):
        """Batches of the stream `seed` jumped `jumps` times (a scan's point)."""
        acc = self.pkg.BatchAccumulators(n_batches)
        soa = acc.soa()
        threads = threads or os.cpu_count() or 1
        st = self.L.tpo_run_batches_jumped(ctypes.byref(cfg.c), rng_kind, seed, jumps, first_batch, n_batches,
                                           ctypes.byref(soa), threads)
        assert st == 0, st
        return acc

    def dump_events(self, cfg, rng_kind, seed, first_event, n):
        out = np.zeros(n, self.pkg.DUMP_DTYPE)
        st = self.L.tpo_dump_events(ctypes.byref(cfg.c), rng_kind, seed, first_event, n,
                                    ctypes.c_void_p(out.ctypes.data))
        assert st == 0, st
        return out

    def m2_sums_of(self, cfg, p_out):
        """m2_sums of the photons p_out[n, 3, 4] (one row per event)."""
        p = np.ascontiguousarray(p_out, np.float64)
        out = np.zeros((p.shape[0], 5), np.float64)
        dp = ctypes.POINTER(ctypes.c_double)
        for i in range(p.shape[0]):
            self.L.tpo_m2_sums_of(ctypes.byref(cfg.c), p[i].ctypes.data_as(dp), out[i].ctypes.data_as(dp))
        return out

    def binned(self, cfg, rng_kind, seed, first_batch, n_batches, nx, ny, xr, yr):
        out = np.zeros((nx * ny, 8), np.float64)
        st = self.L.tpo_binned(ctypes.byref(cfg.c), rng_kind, seed, first_batch, n_batches, nx, ny, xr[0], xr[1],
                               yr[0], yr[1], ctypes.c_void_p(out.ctypes.data))
        assert st == 0, st
        return out

    def merge_finalize(self, cfg, acc):
        res = self.pkg.CFinalResults()
        soa = acc.soa()
        st = self.L.tpo_merge_finalize(ctypes.byref(cfg.c), ctypes.byref(soa), acc.n, ctypes.byref(res))
        assert st == 0, st
        return res

    def res_data(self, cfg, res):
        buf = ctypes.create_string_buffer(1 << 16)
        self.L.tpo_format_res_data(ctypes.byref(cfg.c), ctypes.byref(res), buf, len(buf))
        return buf.value.decode()

    def report(self, cfg, res):
        buf = ctypes.create_string_buffer(1 << 16)
        self.L.tpo_format_report(ctypes.byref(cfg.c), ctypes.byref(res), buf, len(buf))
        return buf.value.decode()

    def draws(self, rng_kind, seed, jumps, skip, n):
        out = np.zeros(n, np.float64)
        self.L.tpo_draws(rng_kind, seed, jumps, skip, n, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out

    def xoshiro_state(self, seed, jumps):
        s = (ctypes.c_uint64 * 4)()
        self.L.tpo_xoshiro_state(seed, jumps, s)
        return list(s)

    def ranf_state(self, seed, resets):
        s = (ctypes.c_int32 * 56)()
        self.L.tpo_ranf_state(seed, resets, s)
        return list(s)

    def couplings(self, cfg):
        g = (ctypes.c_double * 3)()
        self.L.tpo_couplings(ctypes.byref(cfg.c), g)
        return list(g)

    def sigma_contribs(self, cfg):
        g = (ctypes.c_double * 5)()
        self.L.tpo_sigma_contribs(ctypes.byref(cfg.c), g)
        return list(g)
