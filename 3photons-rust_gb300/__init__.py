"""Python host mirror of 3photons-rust over the GB300 event kernel.

The reference program (src/main.rs:75-145) reads `valeurs` with
``Configuration::load`` (src/config.rs:57-128), hands the event loop to
``scheduling::run_simulation`` (src/scheduling/mod.rs:31-59), and prints /
writes the results with ``FinalResults::eric``/``fawzi`` and
``output::dump_results`` (src/resfin.rs:66-194, src/output.rs:30-177). This
module offers the same steps under the same names; the event loop runs in
``libtp_gb300.so`` (CUDA kernels for sm_103a behind the C ABI of
include/tp_gpu.h), and everything else calls the library's host functions.

There is no CPU fallback: if the library or a CUDA device is missing, the
GPU entry points raise.
"""
import ctypes
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtp_gb300.so")

# ---- constants of include/tp_gpu.h -------------------------------------
TP_OK = 0
TP_ERR_INVALID = -1
TP_ERR_UNSUPPORTED = -2
TP_ERR_CUDA = -3
TP_ERR_DEVICE = -4
TP_ERR_TIMEOUT = -5
TP_ERR_NO_DEVICE = -6
TP_ERR_IO = -7
TP_BATCH_SIZE = 10000
TP_RNG_RANF = 0
TP_RNG_XOSHIRO256P = 1
TP_MODE_JUMP_PER_BATCH = 0x100
TP_MODE_NO_PHOTON_SORTING = 0x200
TP_MODE_FASTER_EVGEN = 0x400
TP_PREC_FP64 = 0
TP_PREC_FP32_MIXED = 1
RANF_DEFAULT_SEED = 234612947
XOSHIRO_DEFAULT_SEED = 12345

ERROR_NAMES = {
    TP_ERR_INVALID: "invalid argument",
    TP_ERR_UNSUPPORTED: "unsupported",
    TP_ERR_CUDA: "CUDA error",
    TP_ERR_DEVICE: "device error flag",
    TP_ERR_TIMEOUT: "device wait timed out",
    TP_ERR_NO_DEVICE: "no CUDA device",
    TP_ERR_IO: "I/O error",
}


class TPError(RuntimeError):
    """A negative status returned by the library."""

    def __init__(self, code, message=""):
        self.code = code
        super().__init__("%s (%d)%s" % (ERROR_NAMES.get(code, "error"), code, (": " + message) if message else ""))


# ---- ctypes mirrors of the ABI structs -----------------------------------
class CConfig(ctypes.Structure):
    _fields_ = [
        ("num_events", ctypes.c_uint64),
        ("e_total", ctypes.c_double),
        ("beam_photons_cut", ctypes.c_double),
        ("photon_photon_cut", ctypes.c_double),
        ("e_min", ctypes.c_double),
        ("beam_photon_plane_cut", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("alpha_z", ctypes.c_double),
        ("gev2_to_picobarn", ctypes.c_double),
        ("m_z0", ctypes.c_double),
        ("g_z0", ctypes.c_double),
        ("sin2_weinberg", ctypes.c_double),
        ("branching_ep_em", ctypes.c_double),
        ("beta_plus", ctypes.c_double),
        ("beta_minus", ctypes.c_double),
        ("num_bins", ctypes.c_int32),
        ("impr", ctypes.c_int32),
        ("plot", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
    ]


class CBatchSoa(ctypes.Structure):
    _fields_ = [
        ("selected", ctypes.c_void_p),
        ("spm2", ctypes.c_void_p),
        ("vars", ctypes.c_void_p),
        ("sigma", ctypes.c_void_p),
        ("variance", ctypes.c_void_p),
    ]


class CEventDump(ctypes.Structure):
    _fields_ = [
        ("uniforms", ctypes.c_double * 12),
        ("p_out", (ctypes.c_double * 4) * 3),
        ("cut", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("m2_sums", ctypes.c_double * 5),
    ]


class CFinalResults(ctypes.Structure):
    _fields_ = [
        ("selected_events", ctypes.c_uint64),
        ("spm2", (ctypes.c_double * 5) * 2),
        ("vars", (ctypes.c_double * 5) * 2),
        ("sigma", ctypes.c_double),
        ("prec", ctypes.c_double),
        ("variance", ctypes.c_double),
        ("beta_min", ctypes.c_double),
        ("ss_p", ctypes.c_double),
        ("inc_ss_p", ctypes.c_double),
        ("ss_m", ctypes.c_double),
        ("inc_ss_m", ctypes.c_double),
    ]


class CBinning(ctypes.Structure):
    _fields_ = [
        ("n_emax", ctypes.c_int32),
        ("n_cos", ctypes.c_int32),
        ("emax_lo", ctypes.c_double),
        ("emax_hi", ctypes.c_double),
        ("cos_lo", ctypes.c_double),
        ("cos_hi", ctypes.c_double),
    ]


BIN_STRIDE = 8  # raw sums R_0..R_4, events, sum w, sum w^2
THETA = ("beta_plus", "beta_minus", "m_z0", "g_z0")


DUMP_DTYPE = np.dtype(
    [("uniforms", "<f8", (12,)), ("p_out", "<f8", (3, 4)), ("cut", "<i4"), ("reserved", "<i4"), ("m2_sums", "<f8", (5,))]
)
assert DUMP_DTYPE.itemsize == ctypes.sizeof(CEventDump)

_lib = None


def library():
    """Loads libtp_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libtp_gb300.so is missing: run __graft_entry__.build() first")
    lib = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    vp, u64, i32, dbl = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_double
    sig = {
        "tp_create": (vp, [i32, P(ctypes.c_int)]),
        "tp_destroy": (None, [vp]),
        "tp_last_error": (ctypes.c_char_p, [vp]),
        "tp_run_batches": (i32, [vp, P(CConfig), i32, u64, u64, u64, i32, P(CBatchSoa)]),
        "tp_run_batches_async": (i32, [vp, P(CConfig), i32, u64, u64, u64, i32, P(CBatchSoa), vp]),
        "tp_dump_events": (i32, [vp, P(CConfig), i32, u64, u64, u64, vp]),
        "tp_dump_events_prec": (i32, [vp, P(CConfig), i32, u64, u64, u64, i32, vp]),
        "tp_set_events_per_thread": (i32, [vp, i32]),
        "tp_set_occupancy": (i32, [vp, i32, i32]),
        "tp_set_fe_store_cap": (i32, [vp, u64]),
        "tp_get_tuning": (i32, [vp, i32, ctypes.POINTER(i32), ctypes.POINTER(i32)]),
        "tp_profile": (i32, [vp, i32]),
        "tp_profile_read": (i32, [vp, P(ctypes.c_double), P(ctypes.c_uint64), P(ctypes.c_double), P(ctypes.c_uint64)]),
        "tp_probe_fp64": (i32, [vp, P(ctypes.c_double)]),
        "tp_probe_fp32": (i32, [vp, P(ctypes.c_double)]),
        "tp_recheck_count": (i32, [vp, P(ctypes.c_uint64), i32]),
        "tp_fp32_error": (i32, [vp, P(CConfig), i32, u64, u64, u64, P(ctypes.c_double), P(CBatchSoa),
                                P(CBatchSoa)]),
        "tp_run_batches_noalloc": (i32, [P(CConfig), i32, u64, u64, u64, i32, P(CBatchSoa), vp]),
        "tp_run_points": (i32, [vp, ctypes.c_uint32, P(CConfig), P(ctypes.c_uint64), i32, i32,
                                P(ctypes.c_uint64), P(CBatchSoa), u64]),
        "tp_run_points_ranf": (i32, [vp, ctypes.c_uint32, P(CConfig), P(ctypes.c_int32), i32, i32,
                                     P(ctypes.c_uint64), P(CBatchSoa), u64]),
        "tp_autotune": (i32, [vp, P(CConfig), i32, u64, P(ctypes.c_int), P(ctypes.c_double)]),
        "tp_binned_forward": (i32, [vp, P(CConfig), i32, u64, u64, u64, i32, P(CBinning), vp]),
        "tp_binned_adjoint": (i32, [vp, P(CConfig), i32, u64, u64, u64, i32, P(CBinning), vp,
                                    P(ctypes.c_double), P(ctypes.c_double)]),
        "tp_grad": (i32, [vp, P(CConfig), i32, u64, u64, u64, i32, P(CBinning), vp,
                          P(ctypes.c_double), P(ctypes.c_double)]),
        "tp_coupling_factors": (i32, [P(CConfig), P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_double)]),
        "tp_xoshiro_state_at": (i32, [u64, u64, u64, P(ctypes.c_uint64)]),
        "tp_ranf_state_at": (i32, [ctypes.c_int32, u64, P(ctypes.c_int32), P(ctypes.c_int32)]),
        "tp_config_load": (i32, [ctypes.c_char_p, P(CConfig), ctypes.c_char_p, ctypes.c_size_t]),
        "tp_event_weight": (i32, [dbl, P(ctypes.c_double)]),
        "tp_merge_finalize": (i32, [P(CConfig), P(CBatchSoa), u64, P(CFinalResults)]),
        "tp_format_res_data": (i32, [P(CConfig), P(CFinalResults), ctypes.c_char_p, ctypes.c_size_t]),
        "tp_write_res_data": (i32, [P(CConfig), P(CFinalResults), ctypes.c_char_p]),
        "tp_write_res_times": (i32, [P(CConfig), dbl, ctypes.c_char_p, ctypes.c_char_p]),
        "tp_append_pil_mc": (i32, [P(CConfig), P(CFinalResults), ctypes.c_char_p, ctypes.c_char_p]),
        "tp_format_report": (i32, [P(CConfig), P(CFinalResults), ctypes.c_char_p, ctypes.c_size_t]),
    }
    for name, (res, args) in sig.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
    _lib = lib
    return lib


def _check(code, ctx=None):
    if code != TP_OK:
        msg = library().tp_last_error(ctx).decode() if code != TP_OK else ""
        raise TPError(code, msg)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


# ---- Configuration (src/config.rs) ----------------------------------------
class Configuration:
    """The 18 items of `valeurs` (src/config.rs:8-53, read by
    Configuration::load, src/config.rs:57-128)."""

    FIELDS = [f for f, _ in CConfig._fields_ if f != "reserved"]

    def __init__(self, c=None, **kw):
        self.c = c if c is not None else CConfig()
        for k, v in kw.items():
            setattr(self.c, k, v)

    def __getattr__(self, name):
        if name != "c" and name in Configuration.FIELDS:
            return getattr(self.c, name)
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in Configuration.FIELDS:
            setattr(self.c, name, value)
        else:
            object.__setattr__(self, name, value)

    @classmethod
    def load(cls, path="valeurs", echo=True):
        """Configuration::load: parse, echo (like the reference), check."""
        c = CConfig()
        buf = ctypes.create_string_buffer(4096)
        st = library().tp_config_load(path.encode(), ctypes.byref(c), buf, len(buf))
        if echo:
            print(buf.value.decode(), end="")
        _check(st)
        return cls(c)

    @property
    def num_batches(self):
        return (self.c.num_events + TP_BATCH_SIZE - 1) // TP_BATCH_SIZE

    def replace(self, **kw):
        """A copy with some valeurs fields changed (names as in tp_config)."""
        c = CConfig()
        ctypes.pointer(c)[0] = self.c
        fields = {f[0] for f in CConfig._fields_}
        for k, v in kw.items():
            if k not in fields:
                raise AttributeError("tp_config has no field %r" % k)
            setattr(c, k, v)
        return Configuration(c)

    def as_dict(self):
        return {f: getattr(self.c, f) for f in Configuration.FIELDS}


def rng_flags(rng="ranf", jump_per_batch=False, sorting=True, faster_evgen=False):
    """rng_kind of the C ABI for the reference's cargo features: rng
    (`standard-random`), jump_per_batch (`multi-threading,faster-threading`),
    sorting=False (`no-photon-sorting`), faster_evgen (`faster-evgen`)."""
    kind = {"ranf": TP_RNG_RANF, "xoshiro": TP_RNG_XOSHIRO256P, "standard-random": TP_RNG_XOSHIRO256P}[rng]
    if jump_per_batch:
        kind |= TP_MODE_JUMP_PER_BATCH
    if not sorting:
        kind |= TP_MODE_NO_PHOTON_SORTING
    if faster_evgen:
        kind |= TP_MODE_FASTER_EVGEN
    return kind


def default_seed(rng):
    return RANF_DEFAULT_SEED if rng == "ranf" else XOSHIRO_DEFAULT_SEED


# ---- per-batch accumulators ------------------------------------------------
class BatchAccumulators:
    """ResultsAccumulator sums of consecutive batches, structure of arrays
    (src/resacc.rs:18-34): selected[n], spm2[5, n], vars[5, n], sigma[n],
    variance[n]."""

    def __init__(self, n):
        self.n = n
        self.selected = np.zeros(n, np.uint64)
        self.spm2 = np.zeros((5, n), np.float64)
        self.vars = np.zeros((5, n), np.float64)
        self.sigma = np.zeros(n, np.float64)
        self.variance = np.zeros(n, np.float64)

    def soa(self):
        return CBatchSoa(_ptr(self.selected), _ptr(self.spm2), _ptr(self.vars), _ptr(self.sigma), _ptr(self.variance))

    @classmethod
    def concatenate(cls, parts):
        out = cls(sum(p.n for p in parts))
        i = 0
        for p in parts:
            out.selected[i:i + p.n] = p.selected
            out.spm2[:, i:i + p.n] = p.spm2
            out.vars[:, i:i + p.n] = p.vars
            out.sigma[i:i + p.n] = p.sigma
            out.variance[i:i + p.n] = p.variance
            i += p.n
        return out

    def as_array(self):
        """(n, 13) float64 view: selected, spm2[5], vars[5], sigma, variance."""
        return np.concatenate([self.selected[None].astype(np.float64), self.spm2, self.vars,
                               self.sigma[None], self.variance[None]]).T.copy()

    @classmethod
    def from_array(cls, a):
        a = np.asarray(a, np.float64)
        out = cls(a.shape[0])
        out.selected[:] = a[:, 0].astype(np.uint64)
        out.spm2[:] = a[:, 1:6].T
        out.vars[:] = a[:, 6:11].T
        out.sigma[:] = a[:, 11]
        out.variance[:] = a[:, 12]
        return out


# ---- FinalResults (src/resfin.rs) -------------------------------------------
class FinalResults:
    def __init__(self, cfg, c):
        self.cfg = cfg
        self.c = c
        self.selected_events = c.selected_events
        self.spm2 = np.array([[c.spm2[s][k] for k in range(5)] for s in range(2)])
        self.vars = np.array([[c.vars[s][k] for k in range(5)] for s in range(2)])
        for f in ("sigma", "prec", "variance", "beta_min", "ss_p", "inc_ss_p", "ss_m", "inc_ss_m"):
            setattr(self, f, getattr(c, f))

    def report(self):
        """"IBegin" + eric() + fawzi() text (src/resfin.rs:66-194)."""
        buf = ctypes.create_string_buffer(1 << 16)
        n = library().tp_format_report(ctypes.byref(self.cfg.c), ctypes.byref(self.c), buf, len(buf))
        if n < 0:
            _check(n)
        return buf.value.decode()

    def res_data(self):
        buf = ctypes.create_string_buffer(1 << 16)
        n = library().tp_format_res_data(ctypes.byref(self.cfg.c), ctypes.byref(self.c), buf, len(buf))
        if n < 0:
            _check(n)
        return buf.value.decode()


def merge_finalize(cfg, acc):
    """ResultsAccumulator::merge in batch order, then ::finalize."""
    res = CFinalResults()
    soa = acc.soa()
    _check(library().tp_merge_finalize(ctypes.byref(cfg.c), ctypes.byref(soa), acc.n, ctypes.byref(res)))
    return FinalResults(cfg, res)


# ---- the GPU event loop ------------------------------------------------------
class Context:
    """One CUDA device context (tp_create / tp_destroy)."""

    def __init__(self, device=0):
        lib = library()
        st = ctypes.c_int(0)
        self.h = lib.tp_create(device, ctypes.byref(st))
        if not self.h:
            raise TPError(st.value, lib.tp_last_error(None).decode())
        self.device = device

    def close(self):
        if self.h:
            library().tp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def check(self, code):
        if code != TP_OK:
            raise TPError(code, library().tp_last_error(self.h).decode())

    def set_events_per_thread(self, ept):
        self.check(library().tp_set_events_per_thread(self.h, ept))

    def set_occupancy(self, precision, min_ctas_per_sm):
        """xoshiro event kernel variant of `precision`: 2 or 3 CTAs per SM."""
        self.check(library().tp_set_occupancy(self.h, precision, min_ctas_per_sm))

    def set_fe_store_cap(self, nbytes):
        """Device memory faster-evgen one-stream runs may keep between their
        boundary passes (0: recompute instead)."""
        self.check(library().tp_set_fe_store_cap(self.h, nbytes))

    def tuning(self, precision):
        """(events per thread, kernel variant) in use for `precision`."""
        ept, occ = ctypes.c_int(), ctypes.c_int()
        self.check(library().tp_get_tuning(self.h, precision, ctypes.byref(ept), ctypes.byref(occ)))
        return ept.value, occ.value

    def profile(self, enable=True):
        self.check(library().tp_profile(self.h, 1 if enable else 0))

    def profile_read(self):
        """(event-kernel ms, launches, seed-kernel ms, launches) since profile(True)."""
        em, el, sm, sl = ctypes.c_double(), ctypes.c_uint64(), ctypes.c_double(), ctypes.c_uint64()
        self.check(library().tp_profile_read(self.h, ctypes.byref(em), ctypes.byref(el), ctypes.byref(sm),
                                             ctypes.byref(sl)))
        return em.value, el.value, sm.value, sl.value

    def probe_fp64(self):
        """{'dfma_flops': flop/s, 'log'|'sincos'|'sqrt'|'div': DFMA-equivalents}."""
        out = (ctypes.c_double * 5)()
        self.check(library().tp_probe_fp64(self.h, out))
        return {"dfma_flops": out[0], "log": out[1], "sincos": out[2], "sqrt": out[3], "div": out[4]}

    def probe_fp32(self):
        """{'ffma_flops': FP32 flop/s, 'sfu_ops': special-function operations/s}."""
        out = (ctypes.c_double * 2)()
        self.check(library().tp_probe_fp32(self.h, out))
        return {"ffma_flops": out[0], "sfu_ops": out[1]}

    def fp32_error(self, cfg, first_batch, n_batches, rng="ranf", seed=None, jump_per_batch=False, sorting=True):
        """Per-batch relative error of the FP32-mixed sums against FP64 on the
        same events (-1 where the selected counts differ), and both runs'
        accumulators: (err[n], fp32, fp64)."""
        seed = default_seed(rng) if seed is None else seed
        err = np.zeros(n_batches, np.float64)
        a32, a64 = BatchAccumulators(n_batches), BatchAccumulators(n_batches)
        s32, s64 = a32.soa(), a64.soa()
        self.check(library().tp_fp32_error(self.h, ctypes.byref(cfg.c), rng_flags(rng, jump_per_batch, sorting), seed,
                                           first_batch, n_batches, err.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                           ctypes.byref(s32), ctypes.byref(s64)))
        return err, a32, a64

    def recheck_count(self, reset=True):
        """Events the FP32-mixed path settled with its FP64 recheck."""
        n = ctypes.c_uint64()
        self.check(library().tp_recheck_count(self.h, ctypes.byref(n), 1 if reset else 0))
        return n.value

    def run_batches(self, cfg, first_batch, n_batches, rng="ranf", seed=None, jump_per_batch=False, sorting=True,
                    precision=TP_PREC_FP64, out=None, faster_evgen=False):
        """Per-batch accumulators of batches [first_batch, first_batch + n)."""
        seed = default_seed(rng) if seed is None else seed
        acc = out if out is not None else BatchAccumulators(n_batches)
        soa = acc.soa()
        flags = rng_flags(rng, jump_per_batch, sorting, faster_evgen)
        self.check(library().tp_run_batches(self.h, ctypes.byref(cfg.c), flags,
                                            seed, first_batch, n_batches, precision, ctypes.byref(soa)))
        return acc

    def run_batches_device(self, cfg, first_batch, n_batches, out_ptrs, stream=0, rng="ranf", seed=None,
                           jump_per_batch=False, sorting=True, precision=TP_PREC_FP64, faster_evgen=False):
        """Queues the batches on `stream` writing DEVICE arrays given as five
        raw pointers (selected, spm2, vars, sigma, variance)."""
        seed = default_seed(rng) if seed is None else seed
        soa = CBatchSoa(*[ctypes.c_void_p(p) for p in out_ptrs])
        flags = rng_flags(rng, jump_per_batch, sorting, faster_evgen)
        self.check(library().tp_run_batches_async(self.h, ctypes.byref(cfg.c), flags,
                                                  seed, first_batch, n_batches, precision, ctypes.byref(soa),
                                                  ctypes.c_void_p(stream)))

    def autotune(self, cfg, precision=TP_PREC_FP32_MIXED, sample_batches=2048):
        """Picks events per thread (hence the block shape) for this context."""
        ept, rate = ctypes.c_int(), ctypes.c_double()
        self.check(library().tp_autotune(self.h, ctypes.byref(cfg.c), precision, sample_batches, ctypes.byref(ept),
                                         ctypes.byref(rate)))
        return ept.value, rate.value

    def run_points(self, cfgs, starts, precision=TP_PREC_FP32_MIXED, sorting=True, rng="xoshiro"):
        """Batched form: every point's run in one persistent launch (CUDA
        graph). starts: [n_points, 4] raw xoshiro states, or (rng="ranf")
        [n_points] ranf seeds. Returns one BatchAccumulators per point."""
        n = len(cfgs)
        arr = (CConfig * n)(*[c.c for c in cfgs])
        total = sum((c.num_events + TP_BATCH_SIZE - 1) // TP_BATCH_SIZE for c in cfgs)
        acc = BatchAccumulators(total)
        unit0 = np.zeros(n + 1, np.uint64)
        soa = acc.soa()
        flags = 0 if sorting else TP_MODE_NO_PHOTON_SORTING
        u0 = unit0.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
        if rng == "ranf":
            st = np.ascontiguousarray(starts, np.int32).reshape(n)
            self.check(library().tp_run_points_ranf(self.h, n, arr, st.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                    flags, precision, u0, ctypes.byref(soa), total))
        else:
            st = np.ascontiguousarray(starts, np.uint64).reshape(n, 4)
            self.check(library().tp_run_points(self.h, n, arr, st.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                                               flags, precision, u0, ctypes.byref(soa), total))
        out = []
        for p in range(n):
            a, b = int(unit0[p]), int(unit0[p + 1])
            part = BatchAccumulators(b - a)
            part.selected[:] = acc.selected[a:b]
            part.spm2[:] = acc.spm2[:, a:b]
            part.vars[:] = acc.vars[:, a:b]
            part.sigma[:] = acc.sigma[a:b]
            part.variance[:] = acc.variance[a:b]
            out.append(part)
        return out

    def binned_forward(self, cfg, first_batch, n_batches, binning, seed=XOSHIRO_DEFAULT_SEED,
                       precision=TP_PREC_FP64, jump_per_batch=False, rng="xoshiro"):
        """Per-bin sums [n_bins, 8]: raw R_0..R_4, events, sum w, sum w^2."""
        nb = binning.n_emax * binning.n_cos
        out = np.zeros((nb, BIN_STRIDE), np.float64)
        self.check(library().tp_binned_forward(self.h, ctypes.byref(cfg.c), rng_flags(rng, jump_per_batch),
                                               seed, first_batch, n_batches, precision, ctypes.byref(binning),
                                               ctypes.c_void_p(out.ctypes.data)))
        return out

    def binned_adjoint(self, cfg, first_batch, n_batches, binning, bin_weight, seed=XOSHIRO_DEFAULT_SEED,
                       precision=TP_PREC_FP64, jump_per_batch=False, rng="xoshiro"):
        """(g, s): g_c = sum_e r[bin(e)] raw_c,e, s_c = sum_e raw_c,e."""
        w = np.ascontiguousarray(bin_weight, np.float64)
        g = (ctypes.c_double * 5)()
        sm = (ctypes.c_double * 5)()
        self.check(library().tp_binned_adjoint(self.h, ctypes.byref(cfg.c), rng_flags(rng, jump_per_batch),
                                               seed, first_batch, n_batches, precision, ctypes.byref(binning),
                                               ctypes.c_void_p(w.ctypes.data), g, sm))
        return np.array(g[:]), np.array(sm[:])

    def grad(self, cfg, first_batch, n_batches, binning, bin_weight, seed=XOSHIRO_DEFAULT_SEED,
             precision=TP_PREC_FP64, jump_per_batch=False, rng="xoshiro"):
        """tp_grad: (d lnL/dtheta, d sigma/dtheta) for theta = (beta+, beta-,
        M_Z, Gamma_Z), r = bin_weight = d lnL / d mu per bin."""
        w = np.ascontiguousarray(bin_weight, np.float64)
        dl = (ctypes.c_double * 4)()
        ds = (ctypes.c_double * 4)()
        self.check(library().tp_grad(self.h, ctypes.byref(cfg.c), rng_flags(rng, jump_per_batch), seed,
                                     first_batch, n_batches, precision, ctypes.byref(binning),
                                     ctypes.c_void_p(w.ctypes.data), dl, ds))
        return np.array(dl[:]), np.array(ds[:])

    def dump_events(self, cfg, first_event, n, rng="ranf", seed=None, jump_per_batch=False, sorting=True,
                    precision=TP_PREC_FP64):
        seed = default_seed(rng) if seed is None else seed
        out = np.zeros(n, DUMP_DTYPE)
        self.check(library().tp_dump_events_prec(self.h, ctypes.byref(cfg.c), rng_flags(rng, jump_per_batch, sorting),
                                                 seed, first_event, n, precision, ctypes.c_void_p(out.ctypes.data)))
        return out


def coupling_factors(cfg):
    """(K[5], dK[5, 4], flux): K_c(theta), dK_c/d(beta+, beta-, M_Z, Gamma_Z)."""
    k = (ctypes.c_double * 5)()
    dk = (ctypes.c_double * 20)()
    flux = ctypes.c_double()
    _check(library().tp_coupling_factors(ctypes.byref(cfg.c), k, dk, ctypes.byref(flux)))
    return np.array(k[:]), np.array(dk[:]).reshape(5, 4), flux.value


def binning(n_emax=20, n_cos=20, emax=(0.0, 0.0), cos=(0.0, 0.0)):
    """E of the most energetic photon x cos(it, e- beam); (0, 0) ranges mean
    [sqrt(s)/3, sqrt(s)/2] and [-ACUT, ACUT]."""
    return CBinning(n_emax, n_cos, emax[0], emax[1], cos[0], cos[1])


class BinnedGaussianLikelihood:
    """ln L(theta) = -1/2 sum_b (mu_b(theta) - d_b)^2 / v_b, the binned
    Gaussian log-likelihood of a model run against pseudo-data.

    mu_b(theta) = flux sum_{e in b} w_e(theta) over the model's events; the
    data histogram d_b (and its variance v_b = flux^2 sum w^2, from the data
    run) comes from another run, e.g. at other couplings and another seed.
    theta = (beta+, beta-, M_Z, Gamma_Z). Events do not depend on theta
    (only their weights do), so every evaluation reuses the model's seed.

    value(theta): forward pass (events recomputed on the GPU).
    gradient(theta): forward pass, then the adjoint pass with r_b =
    d lnL/d mu_b; returns d lnL/dtheta and d sigma/dtheta.
    analytic_gradient(theta): the same derivatives from the forward pass's
    per-bin raw sums R_bc (mu_b = flux sum_c R_bc K_c(theta)), the reference
    for the adjoint.
    """

    def __init__(self, ctx, cfg, seed, n_batches, data_hist, data_cfg, bins, precision=TP_PREC_FP64, rng="xoshiro"):
        self.ctx, self.cfg, self.seed, self.n_batches = ctx, cfg, seed, n_batches
        self.bins, self.precision, self.rng = bins, precision, rng
        _, _, flux_d = coupling_factors(data_cfg)
        self.data = flux_d * data_hist[:, 6]
        var = flux_d ** 2 * data_hist[:, 7]
        self.var = np.where(var > 0, var, max(var.max(), 1e-300) * 1e-12 + 1e-300)
        self.last_hist = None

    def theta_cfg(self, theta):
        return self.cfg.replace(**dict(zip(THETA, [float(t) for t in theta])))

    def _mu(self, hist, cfg):
        k, dk, flux = coupling_factors(cfg)
        return flux * hist[:, :5] @ k, k, dk, flux

    def value(self, theta):
        cfg = self.theta_cfg(theta)
        hist = self.ctx.binned_forward(cfg, 0, self.n_batches, self.bins, self.seed, self.precision, rng=self.rng)
        self.last_hist = hist
        mu, k, _, flux = self._mu(hist, cfg)
        lnl = -0.5 * float(np.sum((mu - self.data) ** 2 / self.var))
        sigma = flux * float(hist[:, :5].sum(axis=0) @ k)
        return lnl, sigma, mu

    def gradient(self, theta):
        lnl, sigma, mu = self.value(theta)
        cfg = self.theta_cfg(theta)
        r = -(mu - self.data) / self.var
        g, s = self.ctx.binned_adjoint(cfg, 0, self.n_batches, self.bins, r, self.seed, self.precision, rng=self.rng)
        _, dk, flux = coupling_factors(cfg)
        return lnl, flux * g @ dk, sigma, flux * s @ dk

    def analytic_gradient(self, theta, hist=None):
        cfg = self.theta_cfg(theta)
        hist = self.last_hist if hist is None else hist
        mu, k, dk, flux = self._mu(hist, cfg)
        r = -(mu - self.data) / self.var
        R = hist[:, :5]
        return flux * (r @ R) @ dk, flux * R.sum(axis=0) @ dk


def xoshiro_start(seed, jumps128=0, draws=0):
    """Raw xoshiro256+ state: seed_from_u64(seed), then jumps of 2^128."""
    s = (ctypes.c_uint64 * 4)()
    _check(library().tp_xoshiro_state_at(seed, jumps128, draws, s))
    return list(s)


def scan_points(base, n_points=256, seed=12345, rng="xoshiro"):
    """Parameter points of the batched form: sqrt(s) ~ U[200, 2000] GeV,
    E_min ~ U[1, 50] GeV, the |cos| cuts (beam-photon and photon-photon) ~
    U[0.80, 0.99], beta+, beta- ~ U[-1, 1], events ~ log-U[1e6, 1e8], drawn
    with numpy's PCG64(seed); everything else from `base`. Point p's stream
    is the reference's stream jumped p times (RandomGenerator::jump):
    xoshiro256+ seeded with 12345 and jumped p times by 2^128 (starts: raw
    states), or ranf seeded with 234612947 + 123456 p (starts: the seeds)."""
    r = np.random.Generator(np.random.PCG64(seed))
    cfgs, starts = [], []
    for p in range(n_points):
        cut = float(r.uniform(0.80, 0.99))
        cfgs.append(base.replace(e_total=float(r.uniform(200.0, 2000.0)), e_min=float(r.uniform(1.0, 50.0)),
                                 beam_photons_cut=cut, photon_photon_cut=cut,
                                 beta_plus=float(r.uniform(-1.0, 1.0)), beta_minus=float(r.uniform(-1.0, 1.0)),
                                 num_events=int(np.exp(r.uniform(np.log(1e6), np.log(1e8))))))
        if rng == "ranf":
            starts.append(np.int32(np.uint32((RANF_DEFAULT_SEED + 123456 * p) & 0xffffffff).view(np.int32)))
        else:
            starts.append(xoshiro_start(XOSHIRO_DEFAULT_SEED, p))
    return cfgs, np.array(starts, np.int32 if rng == "ranf" else np.uint64)


def fisher_matrix(model, theta, hist=None):
    """Gauss-Newton Fisher matrix J^T V^-1 J of a BinnedGaussianLikelihood,
    J_bj = d mu_b / d theta_j = flux sum_c R_bc dK_c/dtheta_j, from the
    forward pass's per-bin raw sums."""
    cfg = model.theta_cfg(theta)
    hist = model.last_hist if hist is None else hist
    _, dk, flux = coupling_factors(cfg)
    J = flux * hist[:, :5] @ dk
    return J.T @ (J / model.var[:, None])


def fit(model, theta0, steps=200, lr=0.5, free=(0, 1), damping=1e-3, tol=0.0, info=None):
    """Maximises ln L over the parameters `free` (indices into theta) with at
    most `steps` natural-gradient steps: theta += lr (F + damping) ^-1 g,
    where g comes from the forward + adjoint passes on the GPU and F is the
    Gauss-Newton Fisher matrix of the same forward pass. Stops early once a
    step moves every free parameter by less than `tol` of its standard error
    sqrt(diag F^-1) (tol = 0: never). Returns (theta, covariance estimate
    F^-1 at the end); `info`, a dict, receives the steps taken."""
    theta = np.array(theta0, np.float64)
    idx = list(free)
    F = None
    taken = 0
    for _ in range(steps):
        _, g, _, _ = model.gradient(theta)
        F = fisher_matrix(model, theta)[np.ix_(idx, idx)]
        Fd = F + damping * np.trace(F) / len(idx) * np.eye(len(idx))
        step = lr * np.linalg.solve(Fd, g[idx])
        theta[idx] += step
        taken += 1
        if tol > 0 and np.all(np.abs(step) < tol * np.sqrt(np.diag(np.linalg.inv(F)))):
            break
    if info is not None:
        info["steps"] = taken
    return theta, np.linalg.inv(F)


def run_simulation(cfg, rng="ranf", seed=None, jump_per_batch=False, sorting=True, precision=TP_PREC_FP64,
                   device=0, ctx=None, faster_evgen=False):
    """scheduling::run_simulation (src/scheduling/mod.rs:31-59): every batch
    on the GPU, merged in batch order on the host, finalised."""
    own = ctx is None
    ctx = ctx or Context(device)
    try:
        acc = ctx.run_batches(cfg, 0, cfg.num_batches, rng, seed, jump_per_batch, sorting, precision,
                              faster_evgen=faster_evgen)
    finally:
        if own:
            ctx.close()
    return merge_finalize(cfg, acc)


def run_simulation_sharded(cfg, rank, world_size, run_batches, all_gather, **kw):
    """Batch-range sharding over `world_size` processes with no data-path
    collective: rank r integrates batches [lo_r, hi_r); the per-batch
    accumulators (13 numbers per batch) are gathered once and merged in batch
    order, so the result equals the single-process run bit for bit.

    run_batches(first_batch, n) -> BatchAccumulators; all_gather(ndarray) ->
    list of ndarrays, one per rank (e.g. torch.distributed.all_gather_object).
    """
    nb = cfg.num_batches
    lo = nb * rank // world_size
    hi = nb * (rank + 1) // world_size
    part = run_batches(lo, hi - lo) if hi > lo else BatchAccumulators(0)
    parts = [BatchAccumulators.from_array(a) for a in all_gather(part.as_array())]
    return merge_finalize(cfg, BatchAccumulators.concatenate(parts))


def run_simulation_resumable(cfg, checkpoint, run_batches, chunk_batches=1000, run_key=""):
    """Checkpointed run: integrates the batches chunk by chunk and, after
    every chunk, saves the per-batch sums so far to `checkpoint` (an .npz
    path, written atomically). A restarted call resumes at the first missing
    batch: batch b's stream is a pure function of (stream, seed, b), so the
    resumed run equals an uninterrupted one bit for bit.
    run_batches(first_batch, n) -> BatchAccumulators (e.g. a bound
    Context.run_batches). A checkpoint is only resumed by the same
    configuration (every valeurs field) and the same `run_key`, a string the
    caller makes from what run_batches binds (stream, seed, modes,
    precision)."""
    nb = cfg.num_batches
    done = BatchAccumulators(0)
    config_bytes = np.frombuffer(bytes(cfg.c), np.uint8)
    if os.path.exists(checkpoint):
        with np.load(checkpoint) as z:
            if (int(z["num_events"]) != cfg.num_events or "config" not in z
                    or not np.array_equal(z["config"], config_bytes) or str(z["run_key"]) != run_key):
                raise ValueError("checkpoint belongs to another run")
            done = BatchAccumulators.from_array(z["sums"])
    parts = [done]
    first = done.n
    while first < nb:
        n = min(chunk_batches, nb - first)
        parts.append(run_batches(first, n))
        first += n
        acc = BatchAccumulators.concatenate(parts)
        parts = [acc]
        tmp = checkpoint + ".tmp.npz"
        np.savez(tmp, sums=acc.as_array(), num_events=cfg.num_events, config=config_bytes, run_key=run_key)
        os.replace(tmp, checkpoint)
    return merge_finalize(cfg, BatchAccumulators.concatenate(parts))


def dump_results(cfg, res, elapsed_seconds, directory=".", timestamp=None):
    """output::dump_results (src/output.rs:30-177): prints the report and
    writes res.times, res.data and appends pil.mc."""
    print(res.report(), end="")
    lib = library()
    ts = timestamp.encode() if timestamp else None
    _check(lib.tp_write_res_times(ctypes.byref(cfg.c), elapsed_seconds, ts, os.path.join(directory, "res.times").encode()))
    _check(lib.tp_write_res_data(ctypes.byref(cfg.c), ctypes.byref(res.c), os.path.join(directory, "res.data").encode()))
    _check(lib.tp_append_pil_mc(ctypes.byref(cfg.c), ctypes.byref(res.c), ts, os.path.join(directory, "pil.mc").encode()))


def main(valeurs="valeurs", directory=".", **kw):
    """main() (src/main.rs:75-145)."""
    cfg = Configuration.load(valeurs)
    t0 = time.perf_counter()
    res = run_simulation(cfg, **kw)
    dump_results(cfg, res, time.perf_counter() - t0, directory)
    return res
