"""Benchmark of the e+e- -> 3 photons event loop on GB300.

Workload (one "step"): the FP64 plain path over 1e9 events = 1e5 batches of
10 000 at sqrt(s) = 1000 GeV (E_min 5 GeV, |cos| cuts 0.95, alpha =
1/137.036, M_Z = 91.187, Gamma_Z = 2.490, sin^2 theta_W = 0.2315,
beta+- = 1), random stream xoshiro256+ seeded with 12345 (the reference's
`standard-random` stream), draws bit-exact to the reference's sequential
stream. The inputs are the configuration and the seed; the outputs are the
13 per-batch sums of every batch.

  value     events/s with the outputs kept on the device (CUDA events on the
            launching stream; L2 flushed between steps by a 256 MiB write)
  e2e       events/s through the public C-ABI call with host output arrays
            (tp_run_batches: launch, run, copy of every batch's sums to host)
  roofline  the event kernel's FP64 work (canonical per-event count, the
            transcendental calls weighted by their measured DFMA cost) per
            second against this GPU's DFMA rate measured here
  cpu_baseline  the CPU restatement of the reference path on the host cores

`--impl reference` times the reference's CPU path instead (the CPU
restatement: the Rust reference cannot be built here) on the same workload.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD_EVENTS = 1_000_000_000
SEED = 12345
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
METRIC = "events/s on 1 GB300: FP32-mixed vs FP64 plain at sigma rel.err<=1e-6; grad/fwd time"


WORKLOAD_VALEURS = os.path.join(ROOT, "tests", "golden", "valeurs_sqrts1000")


def workload_config(tp, events):
    cfg = tp.Configuration.load(WORKLOAD_VALEURS, echo=False)
    return cfg.replace(num_events=events)


class ClockSampler:
    """nvidia-smi samples (every 200 ms) while the timed region runs."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + CLOCK_FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[4:]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        seen = set()
        for _, _, flags in rows:
            for n, f in zip(names, flags[1:]):
                if f.lower() == "active":
                    seen.add(n)
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": sorted(seen), "samples": len(rows)}


def algorithmic_flops_per_event(f_acc, costs):
    """Canonical FP64 work of one event: 177 + 623 f_acc flops (minimal
    operation count of the reference formulas), plus per event 3 log, 3
    sincos, 5 + 3 f_acc sqrt and 2 + 9 f_acc divisions, each weighted by its
    measured cost in DFMA (2 flops) equivalents."""
    w = 177.0 + 623.0 * f_acc
    w += 2.0 * (3 * costs["log"] + 3 * costs["sincos"] + (5 + 3 * f_acc) * costs["sqrt"]
                + (2 + 9 * f_acc) * costs["div"])
    return w


def oracle_workload(tp, events):
    """The CPU restatement and the workload configuration parsed by the
    restatement's own `valeurs` reader: the reference arm maps no product
    library."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import tp_oracle_py

    oracle = tp_oracle_py.Oracle(tp)
    st, cfg, _ = oracle.load(WORKLOAD_VALEURS)
    if st != 0:
        raise RuntimeError("cannot read %s (%d)" % (WORKLOAD_VALEURS, st))
    return oracle, cfg.replace(num_events=events)


def cpu_baseline(tp, events_budget_s=3.0):
    """The CPU restatement (FP64, the same xoshiro stream and physics) on all
    host cores over a bounded sample of the workload's first batches."""
    oracle, cfg = oracle_workload(tp, WORKLOAD_EVENTS)
    threads = os.cpu_count() or 1
    kind = tp.rng_flags("xoshiro")
    nb = max(threads, 8)
    t0 = time.perf_counter()
    oracle.run_batches(cfg, 0, nb, kind, SEED, threads)
    dt = time.perf_counter() - t0
    nb = max(nb, int(nb * events_budget_s / max(dt, 1e-3)))
    t0 = time.perf_counter()
    oracle.run_batches(cfg, 0, nb, kind, SEED, threads)
    dt = time.perf_counter() - t0
    ev = nb * tp.TP_BATCH_SIZE
    # one core as well: the reference's default, sequential scheduler
    nb1 = 4
    t0 = time.perf_counter()
    oracle.run_batches(cfg, 0, nb1, kind, SEED, 1)
    dt1 = time.perf_counter() - t0
    return {"value": ev / dt, "unit": "events/s", "cores": threads, "kind": "port",
            "value_1core": nb1 * tp.TP_BATCH_SIZE / dt1,
            "sample": "first %d batches (%d events) of the workload, FP64, %d threads; one core: first %d batches"
                      % (nb, ev, threads, nb1)}


# DFMA-equivalent cost of CUDA 13.0's own FP64 log, sincos, sqrt and
# division on GB300, measured once (8 independent chains per thread at full
# occupancy against 16-chain DFMA, the method of tp_probe_fp64; DFMA rate
# 1.058e12 flop/s) and frozen here, so that a cheaper implementation in the
# kernel raises frac_fixed instead of lowering the work it is credited with.
FROZEN_LIBM_COST = {"log": 30.23, "sincos": 24.94, "sqrt": 8.62, "div": 8.61}


def fixed_fp64_fraction(torch, dev, f_acc, kernel_events_per_s, clocks):
    """The FP64 roofline with every weight fixed: the canonical work of an
    event with each library call at CUDA's own cost (FROZEN_LIBM_COST),
    against the nominal FP64 peak of the GPU, 2 DFMA (4 flops) per clock and
    SM, at the SM clock sampled during the timed region."""
    if FROZEN_LIBM_COST["log"] is None or not clocks.get("sm_mhz"):
        return None
    w = algorithmic_flops_per_event(f_acc, FROZEN_LIBM_COST)
    peak = 4.0 * torch.cuda.get_device_properties(dev).multi_processor_count * clocks["sm_mhz"] * 1e6
    return {"frac": w * kernel_events_per_s / peak, "flops_per_event": w, "peak_tflops": peak / 1e12,
            "weights": dict(FROZEN_LIBM_COST), "peak_source": "nominal 2 DFMA/clock/SM at the sampled SM clock"}


def sig(x, n=5):
    """x with floats rounded to n significant digits (recursively)."""
    if isinstance(x, float):
        return float("%.*g" % (n, x)) if np.isfinite(x) else None
    if isinstance(x, dict):
        return {k: sig(v, n) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [sig(v, n) for v in x]
    return x


def compact_line(d, detail_path=None):
    """The one JSON line bench.py prints: the contract's keys, the legs'
    headline figures, and last (so that a tail of the output keeps them)
    the precision form's events/s, its end-to-end rate, its ratio to the FP64
    path, its largest res.data error against FP64 and the grad/fwd ratio.
    Everything else goes to the --detail file."""
    keep = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "gpu_launches")
    out = {k: d[k] for k in keep if k in d}
    c = d["config"]
    out["config"] = {"workload": "FP64 plain, sqrt(s)=1000 GeV, xoshiro256+ seed 12345 with jump-ahead, 1e9 events "
                                 "= 1e5 batches of 1e4 per GPU", "l2": c["l2"], "parallelism": c["parallelism"],
                     "ept": c["autotuned_events_per_thread"], "ctas_per_sm": c["kernel_variant_ctas_per_sm"]}
    r = d["roofline"]
    ff = r.get("frac_fixed")
    out["roofline"] = {"bound": r["bound"], "achieved": r["achieved"], "peak": r["peak"], "unit": r["unit"],
                       "frac": r["frac"], "traffic": r["traffic"], "kernel": r["kernel"],
                       "peak_source": "DFMA rate measured in this run",
                       "frac_fixed": ff["frac"] if ff else None, "fp64_pipe_active_ncu": r.get("fp64_pipe_active_ncu")}
    if "cpu_baseline" in d:
        cb = d["cpu_baseline"]
        out["cpu_baseline"] = {"value": cb["value"], "unit": cb["unit"], "cores": cb["cores"], "kind": cb["kind"],
                               "value_1core": cb.get("value_1core"), "sample": cb["sample"]}
    out["clocks"] = d["clocks"]
    out["e2e"] = d["e2e"]
    f = d["fp32_mixed"]
    out["fp32"] = {"kernel": f["kernel"], "kernel_ms": f["kernel_ms"], "ept": f["autotuned_events_per_thread"],
                   "ctas_per_sm": f["kernel_variant_ctas_per_sm"], "rechecked": f["rechecked_fraction"],
                   "roofline_frac": f["roofline"]["frac"], "sfu_frac": f["roofline"]["sfu_frac"],
                   "issue_frac": f["roofline"].get("issue", {}).get("frac"),
                   "e2e_bytes": [f["e2e"]["h2d_bytes_per_step"], f["e2e"]["d2h_bytes_per_step"]] if "e2e" in f
                   else None}
    acc = f.get("accuracy_vs_fp64")
    if acc:
        out["fp32"]["selected_equal"] = acc["selected_equal"]
        out["fp32"]["rel_err"] = {k: acc["rel_err"][k] for k in ("sigma", "beta_min", "spm2_1_A", "spm2_1_B+")}
    g = d.get("grad")
    if g:
        t = g["at_test_point"]
        out["grad"] = {"forward_ms": g["forward_ms"], "adjoint_ms": g["adjoint_ms"], "theta": t["theta"],
                       "dlnL_dtheta": t["dlnL_dtheta"], "rel_dev_vs_analytic": t["max_rel_dev_vs_analytic"],
                       "rel_dev_vs_central_diff": t["max_rel_dev_vs_central_diff"]}
        if "flipped_bins" in g:
            out["grad"]["flipped_bins"] = g["flipped_bins"]
        if "fit" in g:
            out["grad"]["fit_beta"] = g["fit"]["beta"]
            out["grad"]["fit_err"] = g["fit"]["beta_err"]
    for key in ("batched", "ranf"):
        if key in d:
            out[key] = {k: v for k, v in d[key].items() if k in ("value", "e2e", "events_per_step", "fp64", "fp32",
                                                                 "fp32_over_xoshiro")}
    if "faster_evgen" in d:
        out["faster_evgen"] = {"%s_%s" % (x["rng"], x.get("precision", "fp64")):
                               {"events_per_s": x["events_per_s"], "boundary_ms": x["boundary_pass_ms"],
                                "ms": x["ms_per_step"]} for x in d["faster_evgen"]}
    out["detail"] = detail_path
    out["fp32_mixed_value"] = f["value"]
    out["fp32_mixed_e2e"] = f["e2e"]["value"] if "e2e" in f else None
    out["fp32_over_fp64"] = f.get("ratio_vs_fp64")
    out["fp32_max_rel_err"] = acc["max_rel_err"] if acc else None
    out["grad_over_fwd"] = g["grad_over_fwd"] if g else None
    value, e2e = out["value"], dict(out["e2e"])
    out = sig(out)
    out["value"], out["e2e"] = value, e2e
    return out


RES_FIELDS = ("sigma", "prec", "beta_min", "ss_p", "inc_ss_p", "ss_m", "inc_ss_m")


def precision_report(r32, r64):
    """Relative error of every res.data quantity of the FP32-mixed path
    against the FP64 path on the same events, next to its statistical error.
    The interference (mixed) contributions are measured on the larger of
    their own size and their natural scale sqrt(|A| |B+|) of the same spin
    (they are statistically zero at sqrt(s) = M_Z)."""
    out = {}
    for f in RES_FIELDS:
        a, b = getattr(r32, f), getattr(r64, f)
        out[f] = abs(a - b) / abs(b) if b else abs(a - b)
    names = ["A", "B+", "B-", "Re_mixed", "Im_mixed"]
    for s in range(2):
        for c in range(5):
            a, b = r32.spm2[s, c], r64.spm2[s, c]
            scale = abs(b) if c < 3 else max(abs(b), float(np.sqrt(abs(r64.spm2[s, 0] * r64.spm2[s, 1]))))
            out["spm2_%d_%s" % (s + 1, names[c])] = abs(a - b) / scale if scale else abs(a - b)
    stat = {"sigma": r64.prec}
    for s in range(2):
        for c in range(3):
            stat["spm2_%d_%s" % (s + 1, names[c])] = float(r64.vars[s, c])
    return out, stat


def issue_roofline(torch, dev, fp32, clocks):
    """The FP32-mixed kernel is issue-bound (no pipe saturated): its second
    roofline is warp instructions issued per second against the schedulers'
    ceiling (4 per SM per clock at the SM clock sampled in this run). The
    kernel's warp instructions per event come from its ncu capture
    (profiles/issue.json); the rate is this run's."""
    path = os.path.join(ROOT, "profiles", "issue.json")
    if not os.path.exists(path) or not clocks.get("sm_mhz") or "kernel_events_per_s" not in fp32:
        return
    prof = json.load(open(path))
    peak = torch.cuda.get_device_properties(dev).multi_processor_count * 4 * clocks["sm_mhz"] * 1e6
    # the count of the variant this run used (the variants spill differently)
    per_event = prof.get("by_variant", {}).get(str(fp32.get("kernel_variant_ctas_per_sm")),
                                              prof["warp_inst_per_event"])
    achieved = per_event * fp32["kernel_events_per_s"]
    fp32["roofline"]["issue"] = {"achieved": achieved, "peak": peak, "unit": "warp instructions/s",
                                 "frac": achieved / peak, "warp_inst_per_event": per_event,
                                 "source": prof["source"]}


def fp32_leg(tp, ctx, torch, dev, stream, args, events, world, rank, fp64_value, acc64, cfg64, first, nb64):
    """The precision form: FP32 phase space, spinors and amplitudes, FP64 batch
    sums, FP64 recheck of events near a cut boundary, on 1e10 events per GPU
    (1e6 batches). Its accuracy is measured on the FP64 leg's 1e9 events."""
    ev32 = 10 * events
    nb = (ev32 + tp.TP_BATCH_SIZE - 1) // tp.TP_BATCH_SIZE
    cfg = workload_config(tp, ev32 * world)
    # events per thread and kernel variant from the autotuner (first 16384
    # batches of this workload); single-leg profiling runs take them from
    # --ept / --occupancy instead
    tuned_ept = ctx.autotune(cfg, tp.TP_PREC_FP32_MIXED, 16384)[0] if not args.only else None
    first32 = rank * nb
    sel = torch.zeros(nb, dtype=torch.int64, device=dev)
    f = torch.zeros(12 * nb, dtype=torch.float64, device=dev)
    ptrs = [sel.data_ptr(), f.data_ptr(), f.data_ptr() + 5 * nb * 8, f.data_ptr() + 10 * nb * 8,
            f.data_ptr() + 11 * nb * 8]

    def step():
        ctx.run_batches_device(cfg, first32, nb, ptrs, stream=stream.cuda_stream, rng="xoshiro", seed=SEED,
                               precision=tp.TP_PREC_FP32_MIXED)

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            step()
    torch.cuda.synchronize()
    ctx.recheck_count(reset=True)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ctx.profile(True)
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            starts[k].record(stream)
            step()
            ends[k].record(stream)
    torch.cuda.synchronize()
    ev_ms, ev_launches, seed_ms, seed_launches = ctx.profile_read()
    ctx.profile(False)
    rechecked = ctx.recheck_count(reset=True)
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    value = world * ev32 * args.steps / (sum(step_ms) * 1e-3)
    out = {"value": value, "unit": "events/s", "events_per_step": ev32 * world, "ms_per_step": sum(step_ms) / len(step_ms),
           "autotuned_events_per_thread": tuned_ept,
           "kernel_variant_ctas_per_sm": ctx.tuning(tp.TP_PREC_FP32_MIXED)[1],
           "kernel": "k_events_xoshiro_fp32", "kernel_ms": ev_ms / args.steps,
           "gpu_launches": int(ev_launches + seed_launches), "ratio_vs_fp64": None,
           "rechecked_fraction": rechecked / (ev32 * args.steps)}
    if fp64_value:
        out["ratio_vs_fp64"] = value / fp64_value
    else:
        del out["ratio_vs_fp64"]
    if not args.only:
        # end to end through the public API (tp_run_batches: host output
        # arrays, their copies in the timed region)
        acc = tp.BatchAccumulators(nb)
        ctx.run_batches(cfg, first32, nb, rng="xoshiro", seed=SEED, precision=tp.TP_PREC_FP32_MIXED, out=acc)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ctx.run_batches(cfg, first32, nb, rng="xoshiro", seed=SEED, precision=tp.TP_PREC_FP32_MIXED, out=acc)
        e2e_s = time.perf_counter() - t0
        out["e2e"] = {"value": world * ev32 * args.steps / e2e_s, "unit": "events/s",
                      "h2d_bytes_per_step": ctypes.sizeof(tp.CConfig), "d2h_bytes_per_step": nb * 13 * 8}
    # roofline: t_min per event = max(W / P_fp32, N_sfu / P_sfu), with the
    # canonical FP work W and special-function count N of an event and the
    # FFMA and MUFU rates measured in this run (tp_probe_fp32)
    rates = ctx.probe_fp32()
    f_acc = float(sel.sum().item()) / ev32
    w = 177.0 + 623.0 * f_acc
    n_sfu = 9.0 + (5.0 + 3.0 * f_acc) + (2.0 + 9.0 * f_acc)
    kernel_rate = ev32 * args.steps / (ev_ms * 1e-3)
    t_fp, t_sfu = w / rates["ffma_flops"], n_sfu / rates["sfu_ops"]
    out["kernel_events_per_s"] = kernel_rate
    out["roofline"] = {"bound": "fp32" if t_fp >= t_sfu else "sfu", "achieved": w * kernel_rate / 1e12,
                       "peak": rates["ffma_flops"] / 1e12, "unit": "TFLOP/s", "frac": max(t_fp, t_sfu) * kernel_rate,
                       "sfu_frac": t_sfu * kernel_rate, "flops_per_event": w, "sfu_ops_per_event": n_sfu,
                       "peak_source": "FFMA and MUFU rates measured in this run (tp_probe_fp32)",
                       "note": "the bit-exact xoshiro256+ stream (integer work) is outside W"}
    if world == 1 and acc64 is not None:
        acc32 = ctx.run_batches(cfg64, first, nb64, rng="xoshiro", seed=SEED, precision=tp.TP_PREC_FP32_MIXED)
        r32 = tp.merge_finalize(cfg64, acc32)
        r64 = tp.merge_finalize(cfg64, acc64)
        err, stat = precision_report(r32, r64)
        out["accuracy_vs_fp64"] = {"events": events, "selected_equal": bool(r32.selected_events == r64.selected_events),
                                   "max_rel_err": max(err.values()), "rel_err": err, "stat_rel_err": stat}
    return out


def gradient_checks(tp, model, theta, h_rel=(1e-2, 1e-2, 1e-4, 1e-2)):
    """The adjoint gradient at `theta` (all four components non-zero away
    from beta+- = 0) against (1) the analytic gradient of the forward pass's
    per-bin raw sums and (2) finite differences of ln L evaluated from the
    same forward pass's per-bin sums, so both references see the same
    events: the five-point stencil (8 D(h) - D(2h)) / 12 h with D(h) = ln
    L(theta + h) - ln L(theta - h) summed bin by bin as (mu+ - mu-)(mu+ +
    mu- - 2 d) / v and mu+ - mu- = flux R (K+ - K-), which avoids the
    cancellation of two large ln L values (or mu values: the A term, most
    of mu, does not depend on M_Z or Gamma_Z). Steps h_i = h_rel[i]
    max(|theta_i|, 1): ln L is a polynomial in beta+- (any step is exact)
    and at sqrt(s) = 1000 GeV mu depends on Gamma_Z only through
    (Gamma_Z / M_Z)^2 next to (s / M_Z^2 - 1)^2 = 1.4e4, so a step of 1e-4
    changes K by 1e-11 relative, below what its rounding resolves: 1e-2
    there; 1e-4 for M_Z. Relative deviations per component."""
    theta = np.array(theta, np.float64)
    _, grad, _, dsigma = model.gradient(theta)
    hist = model.last_hist
    ga, dsa = model.analytic_gradient(theta, hist)

    def dlnl(tp_, tm):
        a, kp, _, flux = model._mu(hist, model.theta_cfg(tp_))
        b, km, _, _ = model._mu(hist, model.theta_cfg(tm))
        # mu+ - mu- from the difference of the coupling factors: the terms
        # that do not depend on theta_i cancel exactly
        dmu = flux * hist[:, :5] @ (kp - km)
        return -0.5 * float(np.sum(dmu * (a + b - 2.0 * model.data) / model.var))

    fd = np.zeros(4)
    for i in range(4):
        e = np.zeros(4)
        e[i] = h_rel[i] * max(abs(theta[i]), 1.0)
        fd[i] = (8.0 * dlnl(theta + e, theta - e) - dlnl(theta + 2 * e, theta - 2 * e)) / (12.0 * e[i])
    rel = lambda a, b: float(np.max(np.abs(a - b) / np.abs(b)))
    return {"theta": theta.tolist(), "dlnL_dtheta": grad.tolist(), "dsigma_dtheta": dsigma.tolist(),
            "max_rel_dev_vs_analytic": rel(grad, ga), "max_rel_dev_dsigma_vs_analytic": rel(dsigma, dsa),
            "max_rel_dev_vs_central_diff": rel(grad, fd),
            "central_diff": "five-point, h_i = %s max(|theta_i|, 1)" % list(h_rel)}


def grad_leg(tp, ctx, args, events, fit_steps=200):
    """The differentiation form: a 20 x 20 binned Gaussian log-likelihood of
    a model run (beta+- = 0, M_Z = 91.187, Gamma_Z = 2.490, seed 12345)
    against pseudo-data (beta+ = 0.3, beta- = -0.2, seed 777), 1e9 events
    each, FP32-mixed. Times the forward pass (value) and the adjoint pass,
    i.e. d(lnL, sigma)/d(beta+, beta-, M_Z, Gamma_Z) by recomputing every
    event from its stream position, then recovers beta+- with `fit_steps`
    gradient steps."""
    prec = tp.TP_PREC_FP32_MIXED
    nb = (events + tp.TP_BATCH_SIZE - 1) // tp.TP_BATCH_SIZE
    bins = tp.binning(20, 20)
    data_cfg = workload_config(tp, events).replace(beta_plus=0.3, beta_minus=-0.2)
    data = ctx.binned_forward(data_cfg, 0, nb, bins, 777, prec)
    model_cfg = workload_config(tp, events).replace(beta_plus=0.0, beta_minus=0.0)
    model = tp.BinnedGaussianLikelihood(ctx, model_cfg, SEED, nb, data, data_cfg, bins, prec)
    theta = (0.0, 0.0, 91.187, 2.49)
    lnl, sigma, mu = model.value(theta)
    r = -(mu - model.data) / model.var
    cfg = model.theta_cfg(theta)
    ctx.binned_adjoint(cfg, 0, nb, bins, r, SEED, prec)  # warm-up
    fwd, adj = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        model.value(theta)
        fwd.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        g, s = ctx.binned_adjoint(cfg, 0, nb, bins, r, SEED, prec)
        adj.append(time.perf_counter() - t0)
    _, dk, flux = tp.coupling_factors(cfg)
    ga, dsa = model.analytic_gradient(theta)
    grad = flux * g @ dk
    f, a = sum(fwd) / len(fwd), sum(adj) / len(adj)
    out = {"events": events, "precision": "fp32_mixed", "bins": "20x20", "forward_ms": 1e3 * f,
           "adjoint_ms": 1e3 * a, "grad_over_fwd": a / f, "gradient_step_over_fwd": (f + a) / f,
           "dlnL_dtheta": grad.tolist(), "dsigma_dtheta": (flux * s @ dk).tolist(),
           "max_rel_dev_vs_analytic": float(np.max(np.abs(grad - ga)) / np.max(np.abs(ga)))}
    out["at_test_point"] = gradient_checks(tp, model, (0.25, -0.1, 91.187, 2.49))
    # the FP32-mixed bins against an FP64 forward pass over the same events:
    # events that changed bin (certified binning: none)
    h64 = ctx.binned_forward(model.theta_cfg(theta), 0, nb, bins, SEED, tp.TP_PREC_FP64)
    h32 = model.last_hist
    out["flipped_bins"] = int(np.abs(h32[:, 5] - h64[:, 5]).sum() // 2)
    if fit_steps:
        # recover beta+- from the pseudo-data: natural-gradient steps, each a
        # forward and an adjoint pass over all events. Only beta-^2 enters the
        # weights, so the start is off beta- = 0 (where d/dbeta- vanishes) and
        # beta- is recovered up to its sign. All fit_steps steps run (the
        # workload's 200), although the fit converges in about 20.
        t0 = time.perf_counter()
        info = {}
        theta_fit, cov = tp.fit(model, (0.1, -0.1, 91.187, 2.49), steps=fit_steps, info=info)
        wall = time.perf_counter() - t0
        err = np.sqrt(np.diag(cov))
        truth = np.array([0.3, -0.2])
        out["fit"] = {"steps": info["steps"], "start": [0.1, -0.1], "truth": truth.tolist(),
                      "beta": theta_fit[:2].tolist(), "beta_err": err.tolist(),
                      "pull": ((theta_fit[:2] - truth) / err).tolist(), "ms_per_step": 1e3 * wall / info["steps"]}
    return out


def faster_evgen_leg(tp, ctx, torch, dev, stream, events, rng, seed, fp64_value=None, precision=0):
    """`--features faster-evgen` (TP_MODE_FASTER_EVGEN), FP64, one stream:
    the boundary pass (chunk maps, host composition, thread start states)
    plus the event kernel, timed on the device around the whole call."""
    cfg = workload_config(tp, events)
    nb = (events + tp.TP_BATCH_SIZE - 1) // tp.TP_BATCH_SIZE
    sel = torch.zeros(nb, dtype=torch.int64, device=dev)
    f = torch.zeros(12 * nb, dtype=torch.float64, device=dev)
    ptrs = [sel.data_ptr(), f.data_ptr(), f.data_ptr() + 5 * nb * 8, f.data_ptr() + 10 * nb * 8,
            f.data_ptr() + 11 * nb * 8]

    def step():
        ctx.run_batches_device(cfg, 0, nb, ptrs, stream=stream.cuda_stream, rng=rng, seed=seed, faster_evgen=True,
                               precision=precision)

    step()
    torch.cuda.synchronize()
    steps = 2
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.profile(True)
    with torch.cuda.stream(stream):
        a.record(stream)
        for _ in range(steps):
            step()
        b.record(stream)
    torch.cuda.synchronize()
    ev_ms, _, _, _ = ctx.profile_read()
    ctx.profile(False)
    ms = a.elapsed_time(b) / steps
    out = {"rng": rng, "precision": "fp32_mixed" if precision else "fp64", "events": events, "ms_per_step": ms,
           "events_per_s": events / (ms * 1e-3),
           "event_kernel_ms": ev_ms / steps, "boundary_pass_ms": ms - ev_ms / steps,
           "selected": int(sel.sum().item())}
    if fp64_value:
        out["vs_default_evgen_fp64"] = out["events_per_s"] / fp64_value
    return out


def ranf_leg(tp, ctx, torch, dev, stream, events, xoshiro_fp32_value):
    """The reference's default stream (ranf, seed 234612947) on the same
    physics, 1e9 events per step, FP64 and FP32-mixed, device-resident
    outputs, CUDA events on the launching stream."""
    cfg = workload_config(tp, events)
    nb = (events + tp.TP_BATCH_SIZE - 1) // tp.TP_BATCH_SIZE
    sel = torch.zeros(nb, dtype=torch.int64, device=dev)
    f = torch.zeros(12 * nb, dtype=torch.float64, device=dev)
    ptrs = [sel.data_ptr(), f.data_ptr(), f.data_ptr() + 5 * nb * 8, f.data_ptr() + 10 * nb * 8,
            f.data_ptr() + 11 * nb * 8]
    out = {"events": events}
    for name, prec in (("fp64", tp.TP_PREC_FP64), ("fp32", tp.TP_PREC_FP32_MIXED)):
        def step():
            ctx.run_batches_device(cfg, 0, nb, ptrs, stream=stream.cuda_stream, rng="ranf",
                                   seed=tp.RANF_DEFAULT_SEED, precision=prec)
        with torch.cuda.stream(stream):
            for _ in range(3):
                step()
        torch.cuda.synchronize()
        steps = 3
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            a.record(stream)
            for _ in range(steps):
                step()
            b.record(stream)
        torch.cuda.synchronize()
        out[name] = events * steps / (a.elapsed_time(b) * 1e-3)
    out["fp32_over_xoshiro"] = out["fp32"] / xoshiro_fp32_value
    return out


def points_leg(tp, ctx, args):
    """The batched form: 256 parameter points (sqrt(s) ~ U[200, 2000] GeV,
    E_min ~ U[1, 50] GeV, |cos| cuts ~ U[0.80, 0.99], beta+- ~ U[-1, 1],
    events ~ log-U[1e6, 1e8], numpy PCG64(12345)), FP32-mixed, in one
    persistent launch replayed from a CUDA graph; events per thread and block
    shape from the autotuner."""
    prec = tp.TP_PREC_FP32_MIXED
    base = workload_config(tp, 1)
    cfgs, starts = tp.scan_points(base, 256, 12345)
    total = sum(c.num_events for c in cfgs)
    ept, tuned_rate = ctx.autotune(base.replace(num_events=163_840_000), prec, 16384)
    ctx.run_points(cfgs, starts, prec)  # captures the graph
    ctx.recheck_count(reset=True)
    ctx.profile(True)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        parts = ctx.run_points(cfgs, starts, prec)
    wall = time.perf_counter() - t0
    graph_ms, launches, _, _ = ctx.profile_read()
    ctx.profile(False)
    res = tp.merge_finalize(cfgs[0], parts[0])
    return {"points": len(cfgs), "events_per_step": total, "precision": "fp32_mixed",
            "value": total * args.steps / (graph_ms * 1e-3), "unit": "events/s",
            "graph_ms_per_step": graph_ms / args.steps, "graph_launches": int(launches),
            "e2e": total * args.steps / wall, "autotuned_events_per_thread": ept,
            "kernel_variant_ctas_per_sm": ctx.tuning(prec)[1],
            "autotune_sample_events_per_s": tuned_rate,
            "min_max_events_per_point": [min(c.num_events for c in cfgs), max(c.num_events for c in cfgs)],
            "rechecked_fraction": ctx.recheck_count(reset=True) / (total * args.steps),
            "point0_sigma_pb": res.sigma}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import __graft_entry__ as graft

    tp = graft.package()  # ctypes struct layouts and constants only: no library load
    oracle, cfg = oracle_workload(tp, WORKLOAD_EVENTS)
    threads = os.cpu_count() or 1
    kind = tp.rng_flags("xoshiro")
    nb = 4 * threads
    for _ in range(args.warmup):
        oracle.run_batches(cfg, 0, nb, kind, SEED, threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.run_batches(cfg, 0, nb, kind, SEED, threads)
        times.append(time.perf_counter() - t0)
    ev = nb * tp.TP_BATCH_SIZE
    value = ev * len(times) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "sqrt(s)=1000 GeV, xoshiro256+ seed 12345, FP64 plain; each step the first "
                               "%d batches (%d events) of the 1e9-event run" % (nb, ev),
                   "same_config": "same physics, stream and metric; each step the first %d batches of the "
                                  "workload, not all 1e5 (a bounded CPU sample)" % nb,
                   "events_per_step": ev, "threads": threads},
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": "port",
                         "sample": "CPU restatement of the reference path (the Rust reference has no toolchain "
                                   "here), %d threads, %d events per step" % (threads, ev)},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours")
    ap.add_argument("--events", type=int, default=WORKLOAD_EVENTS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ept", type=int, default=None, help="with --only: events per thread")
    ap.add_argument("--occupancy", type=int, default=None, help="with --only: kernel variant, CTAs per SM")
    ap.add_argument("--only", choices=["fp64", "fp32", "fe"], default=None,
                    help="time one leg only (no e2e, no CPU baseline): for profiler captures")
    ap.add_argument("--detail", default=None,
                    help="also write every measured quantity (per-quantity errors, fit trace) to this JSON file")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import __graft_entry__ as graft

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    tp = graft.package()
    ctx = tp.Context(local)
    if args.only and args.ept:
        ctx.set_events_per_thread(args.ept)
    if args.only and args.occupancy:
        prec = tp.TP_PREC_FP64 if args.only == "fp64" else tp.TP_PREC_FP32_MIXED
        ctx.set_occupancy(prec, args.occupancy)
    events = args.events
    # weak scaling: every rank integrates its own 1e9-event range of one
    # world * 1e9-event run
    cfg = workload_config(tp, events * world)
    nb = (events + tp.TP_BATCH_SIZE - 1) // tp.TP_BATCH_SIZE
    first = rank * nb
    if args.only == "fp32":
        out = fp32_leg(tp, ctx, torch, torch.device("cuda", local), torch.cuda.Stream(torch.device("cuda", local)),
                       args, events // 10, world, rank, None, None, None, 0, 0)
        if rank == 0:
            print(json.dumps(out))
        return
    if args.only == "fe":
        dev = torch.device("cuda", local)
        st = torch.cuda.Stream(dev)
        out = [faster_evgen_leg(tp, ctx, torch, dev, st, events, "xoshiro", SEED),
               faster_evgen_leg(tp, ctx, torch, dev, st, events // 5, "ranf", tp.RANF_DEFAULT_SEED)]
        if rank == 0:
            print(json.dumps(out))
        return
    costs = ctx.probe_fp64()
    if args.only and args.ept:
        tuned_ept64 = args.ept
    else:
        tuned_ept64, _ = ctx.autotune(cfg, tp.TP_PREC_FP64, 8192)

    dev = torch.device("cuda", local)
    sel = torch.zeros(nb, dtype=torch.int64, device=dev)
    f = torch.zeros(12 * nb, dtype=torch.float64, device=dev)
    ptrs = [sel.data_ptr(), f.data_ptr(), f.data_ptr() + 5 * nb * 8, f.data_ptr() + 10 * nb * 8,
            f.data_ptr() + 11 * nb * 8]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(dev)  # a named stream: the library launches on it

    def step():
        ctx.run_batches_device(cfg, first, nb, ptrs, stream=stream.cuda_stream, rng="xoshiro", seed=SEED)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ctx.profile(True)
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                step()
                ends[k].record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    ev_ms, ev_launches, seed_ms, seed_launches = ctx.profile_read()
    ctx.profile(False)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    if args.only == "fp64":
        if rank == 0:
            print(json.dumps({"leg": "fp64", "events": events, "ms_per_step": sum(step_ms) / len(step_ms),
                              "events_per_s": events * len(step_ms) / (sum(step_ms) * 1e-3)}))
        return
    total_s = sum(step_ms) * 1e-3
    if dist:
        t = torch.tensor([total_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    value = world * events * args.steps / total_s

    selected = int(sel.sum().item())
    f_acc = selected / events
    w = algorithmic_flops_per_event(f_acc, costs)
    launch_ms = ev_ms / max(ev_launches, 1)
    events_per_launch = events * args.steps / max(ev_launches, 1)
    achieved = w * events_per_launch / (launch_ms * 1e-3)
    peak = costs["dfma_flops"]
    traffic = pipe_active = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        tr = json.load(open(tpath))
        if "bytes_per_event" in tr:
            traffic = tr["bytes_per_event"] * events_per_launch
        pipe_active = tr.get("fp64_pipe_active")

    # HBM for scale: the kernel's DRAM traffic per launch (ncu) over its
    # launch time, against the measured copy bandwidth of this GPU model
    hbm = None
    ppath = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if traffic is not None and os.path.exists(ppath):
        hbm_gbs = json.load(open(ppath)).get("hbm_gbs")
        if hbm_gbs:
            got = traffic / (launch_ms * 1e-3) / 1e9
            hbm = {"achieved": got, "peak": hbm_gbs, "unit": "GB/s", "frac": got / hbm_gbs,
                   "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}

    # end to end through the public API: host output arrays, copies included
    acc = tp.BatchAccumulators(nb)
    ctx.run_batches(cfg, first, nb, rng="xoshiro", seed=SEED, out=acc)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx.run_batches(cfg, first, nb, rng="xoshiro", seed=SEED, out=acc)
    e2e_s = time.perf_counter() - t0
    e2e = {"value": world * events * args.steps / e2e_s if world == 1 else events * args.steps / e2e_s * world,
           "unit": "events/s", "h2d_bytes_per_step": ctypes.sizeof(tp.CConfig),
           "d2h_bytes_per_step": nb * 13 * 8}
    sigma = None
    if rank == 0 and world == 1:
        sigma = tp.merge_finalize(cfg, acc).sigma

    fp32 = fp32_leg(tp, ctx, torch, dev, stream, args, events, world, rank, value, acc, cfg, first, nb)

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": sum(step_ms) / len(step_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "FP64 plain path, sqrt(s)=1000 GeV, xoshiro256+ seed 12345 with jump-ahead, "
                               "1e9 events = 1e5 batches of 1e4 per GPU",
                   "events_per_step": events * world, "batches": nb * world, "precision": "fp64",
                   "l2": "flushed between steps (256 MiB write)", "parallelism": "batch-range shards, no collective",
                   "autotuned_events_per_thread": tuned_ept64,
                   "kernel_variant_ctas_per_sm": ctx.tuning(tp.TP_PREC_FP64)[1]},
        "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "DFMA throughput measured in this run (tp_probe_fp64)",
                     "kernel": "k_events_xoshiro_fp64", "flops_per_event": w, "f_acc": f_acc,
                     "dfma_cost": {k: v for k, v in costs.items() if k != "dfma_flops"}, "hbm": hbm,
                     "fp64_pipe_active_ncu": pipe_active},
        "e2e": e2e,
        "gpu_launches": int(ev_launches + seed_launches),
        "kernel_ms": {"events": ev_ms / args.steps, "seed": seed_ms / args.steps},
        "clocks": clocks.summary(),
        "result": {"sigma_pb": sigma, "selected": selected},
        "fp32_mixed": fp32,
    }
    issue_roofline(torch, dev, fp32, line["clocks"])
    line["roofline"]["frac_fixed"] = fixed_fp64_fraction(torch, dev, f_acc, events_per_launch / (launch_ms * 1e-3),
                                                         line["clocks"])
    if world == 1:
        line["grad"] = grad_leg(tp, ctx, args, events)
        line["batched"] = points_leg(tp, ctx, args)
        line["ranf"] = ranf_leg(tp, ctx, torch, dev, stream, events, fp32["value"])
        line["faster_evgen"] = [faster_evgen_leg(tp, ctx, torch, dev, stream, events, "xoshiro", SEED, value),
                                faster_evgen_leg(tp, ctx, torch, dev, stream, events // 5, "ranf",
                                                 tp.RANF_DEFAULT_SEED),
                                faster_evgen_leg(tp, ctx, torch, dev, stream, events, "xoshiro", SEED,
                                                 precision=tp.TP_PREC_FP32_MIXED),
                                faster_evgen_leg(tp, ctx, torch, dev, stream, events // 5, "ranf",
                                                 tp.RANF_DEFAULT_SEED, precision=tp.TP_PREC_FP32_MIXED)]
    if not args.no_cpu_baseline and world == 1:
        line["cpu_baseline"] = cpu_baseline(tp)
    if args.detail:
        with open(args.detail, "w") as fh:
            json.dump(line, fh, indent=1)
    print(json.dumps(compact_line(line, args.detail)))
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
