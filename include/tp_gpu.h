/*
 * tp_gpu.h — C ABI of the GB300 event kernel for e+e- -> 3 photons.
 *
 * This library replaces the per-event loop of 3photons-rust: the scheduler
 * seam `scheduling::run_simulation(num_events, simulate_events)`
 * (src/scheduling/mod.rs:31-59) together with its backends
 * `sequential::run_simulation_impl` (src/scheduling/sequential.rs:15-40) and
 * `multi_threading::run_simulation_impl` (src/scheduling/multi_threading.rs:16-75),
 * and the per-batch closure they call (src/main.rs:103-128):
 * random draws -> RAMBO phase space -> cuts -> spinor products -> helicity
 * amplitudes -> ResultsAccumulator::integrate (src/resacc.rs:121-129).
 *
 * The host keeps the rest of the program: the `valeurs` input
 * (src/config.rs:57-128), the ordered batch merge (src/resacc.rs:133-139),
 * finalisation (src/resacc.rs:142-223) and the res.data / stdout writers
 * (src/output.rs:30-269, src/resfin.rs:66-194).  Those host-side pieces are
 * exported below as well, so a caller in any language can run the whole
 * program through this header.
 *
 * Conventions (every entry point):
 *  - plain pointers and sizes only; no CUDA or torch types in signatures;
 *  - functions return TP_OK (0) on success or a negative TP_ERR_* code and
 *    never abort; the message of the last failure of a context is returned by
 *    tp_last_error();
 *  - one context per host thread; calls are synchronous unless their name
 *    ends in _async;
 *  - device memory is owned by the context (about 35 MiB of tables and
 *    scratch at creation, more for large ranges, binned passes and
 *    faster-evgen), host output buffers by the caller.
 */
#ifndef TP_GPU_H
#define TP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TP_OK 0
#define TP_ERR_INVALID (-1)     /* bad argument or configuration            */
#define TP_ERR_UNSUPPORTED (-2) /* valid request the library does not serve */
#define TP_ERR_CUDA (-3)        /* CUDA allocation / launch / copy failure  */
#define TP_ERR_DEVICE (-4)      /* a kernel raised its device error flag    */
#define TP_ERR_TIMEOUT (-5)     /* a bounded device wait gave up            */
#define TP_ERR_NO_DEVICE (-6)   /* no usable CUDA device                    */
#define TP_ERR_IO (-7)          /* host file input / output failed          */

/* Events per batch: EVENT_BATCH_SIZE (src/scheduling/mod.rs:21). Batch b
 * holds events [b*TP_BATCH_SIZE, min((b+1)*TP_BATCH_SIZE, num_events)). */
#define TP_BATCH_SIZE 10000

/* Number of matrix-element contributions A, B+, B-, Re(mixed), Im(mixed)
 * (src/matelems.rs:21-33). */
#define TP_NUM_CONTRIB 5

/* ---- random streams ------------------------------------------------------
 * rng_kind = one TP_RNG_* value, optionally OR-ed with TP_MODE_* flags.
 *
 * TP_RNG_RANF: Knuth's subtractive generator (src/random/ranf.rs), seed is
 *   the i32 ranf seed (reference default 234612947, ranf.rs:31).
 * TP_RNG_XOSHIRO256P: xoshiro256+ seeded through SplitMix64 from a 64-bit
 *   seed, uniform = (next_u64 >> 11) * 2^-53 (src/random/standard.rs:21-35;
 *   reference default seed 12345).
 *
 * Without flags the whole run is ONE stream consumed 12 draws per event in
 * event order, exactly like the reference's sequential and reproducible
 * multi-threaded schedulers; every batch starts by jump-ahead.
 * TP_MODE_JUMP_PER_BATCH reproduces `--features
 * multi-threading,faster-threading`: batch b starts from the seed jumped b
 * times by RandomGenerator::jump (ranf: reseed with seed+123456*b in i32
 * wrapping arithmetic, ranf.rs:137-140; xoshiro: b jumps of 2^128 draws,
 * standard.rs:53-55).
 * TP_MODE_NO_PHOTON_SORTING reproduces `--features no-photon-sorting`
 * (src/evgen.rs:109, src/event.rs:96-105).
 * TP_MODE_FASTER_EVGEN reproduces `--features faster-evgen`
 * (src/evgen.rs:143-173, 221-249): 9 + 6 draws per event as random_array
 * blocks, plus 2 per re-rolled unit-circle point, so the draws per event
 * vary. The library first finds every event's first draw (a pass over the
 * stream's accept bits from draw 0, also for first_batch > 0), then runs the
 * events, in FP64 or FP32-mixed (the same draws and accept decisions;
 * FP32 physics with the certified cuts), batch
 * accumulators only (tp_run_batches / tp_run_batches_async); the _async call
 * waits for the boundary pass before it queues the event kernels. A
 * one-stream run keeps the pass's accept bits, chases and stream
 * checkpoints in device memory between its two halves (about 16 GB per
 * 1e9 xoshiro events, 12 GB ranf; budget: tp_set_fe_store_cap, default
 * 16 GiB; larger runs recompute them). */
#define TP_RNG_RANF 0
#define TP_RNG_XOSHIRO256P 1
#define TP_RNG_KIND_MASK 0xff
#define TP_MODE_JUMP_PER_BATCH 0x100
#define TP_MODE_NO_PHOTON_SORTING 0x200
#define TP_MODE_FASTER_EVGEN 0x400

#define TP_RANF_DEFAULT_SEED 234612947ull
#define TP_XOSHIRO_DEFAULT_SEED 12345ull

/* ---- precision ---------------------------------------------------------- */
#define TP_PREC_FP64 0       /* FP64 throughout (the reference's default) */
#define TP_PREC_FP32_MIXED 1 /* FP32 event math, FP64 batch sums, FP64
                                recheck of events near a cut boundary     */

/* ---- configuration: the 18 items of `valeurs` (src/config.rs:8-53, read
 * in file order by Configuration::load, src/config.rs:84-101) ------------- */
typedef struct tp_config {
  uint64_t num_events;          /* ITOT: total events of the run; also the
                                   normalisation of every event weight
                                   (src/resacc.rs:83-86)                   */
  double e_total;               /* ETOT, centre-of-mass energy (GeV)      */
  double beam_photons_cut;      /* ACUT, max |cos(photon, beam)|          */
  double photon_photon_cut;     /* BCUT, max cos(photon, photon)          */
  double e_min;                 /* EMIN, min photon energy (GeV)          */
  double beam_photon_plane_cut; /* SINCUT, min cos(beam, plane normal)    */
  double alpha;                 /* fine structure constant                */
  double alpha_z;               /* fine structure constant at the Z peak  */
  double gev2_to_picobarn;      /* CONVERS                                */
  double m_z0;                  /* Z mass (GeV)                           */
  double g_z0;                  /* Z width (GeV)                          */
  double sin2_weinberg;         /* sin^2(theta_W)                         */
  double branching_ep_em;       /* BR(Z -> e+e-)                          */
  double beta_plus;             /* anomalous coupling beta+               */
  double beta_minus;            /* anomalous coupling beta-               */
  int32_t num_bins;             /* NBIN (read, unused by the reference)   */
  int32_t impr;                 /* must be 0 (src/config.rs:120-124)      */
  int32_t plot;                 /* must be 0 (src/config.rs:117)          */
  int32_t reserved;             /* keep 0                                 */
} tp_config;

/* ---- per-batch accumulators: ResultsAccumulator's running sums ---------
 * (src/resacc.rs:18-34). Structure of arrays, every array n_batches long;
 * spm2 and vars are contribution-major: element [k * n_batches + b].      */
typedef struct tp_batch_soa {
  uint64_t *selected; /* events that passed the cuts                 */
  double *spm2;       /* [5][n] sum of per-event |M|^2 contributions  */
  double *vars;       /* [5][n] sum of their squares                  */
  double *sigma;      /* [n]    sum of event weights                  */
  double *variance;   /* [n]    sum of squared event weights          */
} tp_batch_soa;

/* ---- one dumped event (parity checks) ------------------------------------ */
typedef struct tp_event_dump {
  double uniforms[12];    /* the 12 draws, in draw order                 */
  double p_out[3][4];     /* photons after sorting, [photon][X,Y,Z,E]    */
  int32_t cut;            /* 0 kept; 1 energy, 2 beam, 3 pair, 4 plane   */
  int32_t reserved;
  double m2_sums[5];      /* MEsContributions::m2_sums (0 when cut)      */
} tp_event_dump;

/* ---- final results: FinalResults (src/resfin.rs:26-62) ------------------ */
typedef struct tp_final_results {
  uint64_t selected_events;
  double spm2[2][5]; /* [spin][contribution] */
  double vars[2][5];
  double sigma;
  double prec;
  double variance;
  double beta_min;
  double ss_p, inc_ss_p;
  double ss_m, inc_ss_m;
} tp_final_results;

/* ========================================================================
 * GPU context
 * ======================================================================== */
typedef struct tp_ctx tp_ctx;

/* Creates a context on CUDA device `device`. On failure returns NULL and
 * stores a TP_ERR_* code in *status (if non-NULL). */
tp_ctx *tp_create(int device, int *status);
void tp_destroy(tp_ctx *ctx);
/* Message of the last failing call on `ctx` ("" if none). With ctx == NULL:
 * the message of the last failing context-free call (tp_create,
 * tp_run_batches_noalloc) on this thread. */
const char *tp_last_error(const tp_ctx *ctx);

/* Runs batches [first_batch, first_batch + n_batches) of a run configured by
 * `cfg` and writes each batch's accumulators to the caller-owned HOST arrays
 * of `out`. Replaces run_simulation_impl's loop over batches
 * (src/scheduling/sequential.rs:15-40) and the per-batch closure
 * (src/main.rs:103-128); merging in batch order is left to the caller
 * (tp_merge_finalize below), exactly as ResultsAccumulator::merge does.
 * first_batch lets a caller resume or shard a run: batch b's random stream
 * is a pure function of (rng_kind, seed, b). */
int tp_run_batches(tp_ctx *ctx, const tp_config *cfg, int rng_kind,
                   uint64_t seed, uint64_t first_batch, uint64_t n_batches,
                   int precision, tp_batch_soa *out);

/* Same as tp_run_batches, but `out` holds DEVICE pointers and the work is
 * queued on `stream` (a cudaStream_t, NULL = the context's stream) without
 * a host synchronisation. */
int tp_run_batches_async(tp_ctx *ctx, const tp_config *cfg, int rng_kind,
                         uint64_t seed, uint64_t first_batch,
                         uint64_t n_batches, int precision,
                         tp_batch_soa *out, void *stream);

/* Recomputes events [first_event, first_event + n) in FP64 and writes one
 * tp_event_dump per event into the caller's host array (parity checks of
 * single events against the reference's event loop, src/main.rs:108-124). */
int tp_dump_events(tp_ctx *ctx, const tp_config *cfg, int rng_kind,
                   uint64_t seed, uint64_t first_event, uint64_t n,
                   tp_event_dump *out);

/* tp_dump_events for a given precision. With TP_PREC_FP32_MIXED the dump
 * shows the FP32-mixed path's view of each event: FP32 momenta (widened),
 * FP32 m2 sums, and `reserved` = 1 where the FP64 recheck decided the
 * event's cuts. */
int tp_dump_events_prec(tp_ctx *ctx, const tp_config *cfg, int rng_kind,
                        uint64_t seed, uint64_t first_event, uint64_t n,
                        int precision, tp_event_dump *out);

/* Tuning: events each thread integrates in the xoshiro kernels, for both
 * precisions and the binned passes (defaults: 40 for the event kernels,
 * 313 for the binned passes; ceil(10000 / ept) must not exceed 256). No
 * counterpart in the reference, whose batches run on one CPU thread each. */
int tp_set_events_per_thread(tp_ctx *ctx, int ept);

/* Tuning: the xoshiro event kernel variant of `precision`, compiled for 2
 * (default), 3 or (FP32-mixed only) 4 resident CTAs of 256 threads per SM:
 * at most 128, 80 or 64 registers per thread (fewer registers, more
 * resident warps to hide latency, whatever the block shape). Results are
 * the same either way. */
int tp_set_occupancy(tp_ctx *ctx, int precision, int min_ctas_per_sm);

/* Memory: the device memory (bytes) that faster-evgen one-stream runs may
 * keep between their two boundary passes (per chunk of 32 768 draws its
 * accept bits, chases and stream checkpoints; about 16 GB per 1e9 events).
 * Default 16 GiB; a run whose store would not fit computes them a second
 * time instead (slower, same results); 0 never keeps them. No counterpart
 * in the reference. */
int tp_set_fe_store_cap(tp_ctx *ctx, uint64_t bytes);

/* Tuning in use for `precision`: events per thread and kernel variant
 * (minimum resident CTAs per SM), as set or picked by tp_autotune. */
int tp_get_tuning(tp_ctx *ctx, int precision, int *ept, int *min_ctas_per_sm);

/* ---- batched form: many parameter points --------------------------------
 * No counterpart in the reference, which runs one configuration per process.
 * Runs n_points complete runs, each with its own configuration (physics,
 * cuts, couplings, num_events) and its own xoshiro256+ stream given by its
 * raw state at draw 0 (starts[4 p .. 4 p + 3], e.g. from
 * tp_xoshiro_state_at), in ONE persistent launch captured once in a CUDA
 * graph and replayed while the shapes stay the same. Point p's batches are
 * outputs [unit0[p], unit0[p + 1]) of the caller's host arrays (capacity =
 * their length; unit0 has n_points + 1 entries). mode_flags may be
 * TP_MODE_NO_PHOTON_SORTING. Merge and finalise each point's range with
 * tp_merge_finalize. */
int tp_run_points(tp_ctx *ctx, uint32_t n_points, const tp_config *cfgs,
                  const uint64_t *starts, int mode_flags, int precision,
                  uint64_t *unit0, tp_batch_soa *out, uint64_t capacity);

/* tp_run_points on the ranf stream (the reference's default generator):
 * point p's stream is RanfGenerator seeded with seeds[p] (seeded_new,
 * src/random/ranf.rs:36-66), consumed 12 draws per event through the
 * point's batches. A scan that gives point p the reference's p-th jump
 * (RandomGenerator::jump, src/random/ranf.rs:137-140) passes
 * seeds[p] = seed + 123456 p. A seed whose state leaves [0, 1e9) gives
 * TP_ERR_UNSUPPORTED (no jump-ahead). Other arguments as tp_run_points. */
int tp_run_points_ranf(tp_ctx *ctx, uint32_t n_points, const tp_config *cfgs,
                       const int32_t *seeds, int mode_flags, int precision,
                       uint64_t *unit0, tp_batch_soa *out, uint64_t capacity);

/* Autotuner: times the xoshiro event kernel of `precision` on the first
 * `sample_batches` batches of cfg for each candidate events-per-thread
 * (which fixes the block shape, ceil(10000 / ept) threads rounded to
 * warps) and each kernel variant (2 or 3 resident CTAs per SM, and 4 for
 * FP32-mixed), each on a whole number of waves of resident CTAs within
 * the sample; keeps the fastest pair for `precision` in this context (its
 * later launches of that precision: batches, tp_run_points, the binned
 * passes) and reports its events per thread. */
int tp_autotune(tp_ctx *ctx, const tp_config *cfg, int precision,
                uint64_t sample_batches, int *best_ept,
                double *best_events_per_s);

/* ---- binned observables and their adjoint ---------------------------------
 * No counterpart in the reference (its histogram settings `num_bins`/`plot`
 * are read but unused, src/config.rs:45-51, src/main.rs:122). Every kept
 * event has the weight w = sum_c raw_c K_c(theta): raw_c, the five unscaled
 * helicity sums of the event (A, B+, B-, Re and Im of the mixed term,
 * src/matelems.rs:53-86), depend only on its kinematics; K_c, the couplings
 * times the sigma contributions (src/coupling.rs:23-33,
 * src/resacc.rs:59-100), on theta = (beta+, beta-, M_Z, Gamma_Z). Bins:
 * x = energy of the most energetic photon, y = cosine of its angle to the
 * electron beam; bin index ix * n_cos + iy; values outside the range go to
 * the edge bins. Both passes take either stream (rng_kind as for
 * tp_run_batches, TP_MODE_FASTER_EVGEN excepted). TP_PREC_FP32_MIXED bins
 * in FP32 with a certified decision: an event whose FP32 leading-photon
 * energy or cosine lies within its error bound of an inner bin edge is
 * binned from FP64 momenta, so every event lands in the bin of the FP64
 * pass (its sums carry FP32 rounding). */
typedef struct tp_binning {
  int32_t n_emax, n_cos;    /* n_emax * n_cos <= 1024                       */
  double emax_lo, emax_hi;  /* GeV; both 0: [sqrt(s)/3, sqrt(s)/2]           */
  double cos_lo, cos_hi;    /* both 0: [-ACUT, ACUT]                         */
} tp_binning;

/* Forward pass: per bin, 8 sums [raw_0..raw_4, events, w, w^2] (w at the
 * theta of cfg) into the caller's host array of n_emax * n_cos * 8. */
int tp_binned_forward(tp_ctx *ctx, const tp_config *cfg, int rng_kind,
                      uint64_t seed, uint64_t first_batch, uint64_t n_batches,
                      int precision, const tp_binning *bins, double *out);

/* Adjoint pass: recomputes every event from its stream position and returns
 * g_c = sum_e r[bin(e)] raw_c,e and s_c = sum_e raw_c,e, where r is the
 * caller's per-bin weight (for a likelihood L: r_b = d lnL / d mu_b). With
 * flux and dK from tp_coupling_factors: d lnL/dtheta = flux sum_c g_c dK_c,
 * d sigma/dtheta = flux sum_c s_c dK_c. Batches are summed in order. */
int tp_binned_adjoint(tp_ctx *ctx, const tp_config *cfg, int rng_kind,
                      uint64_t seed, uint64_t first_batch, uint64_t n_batches,
                      int precision, const tp_binning *bins,
                      const double *bin_weight, double g[5], double s[5]);

/* The gradient in one call: tp_binned_adjoint composed with
 * tp_coupling_factors, d lnL/dtheta[i] = flux sum_c g_c dK_c/dtheta_i and
 * d sigma/dtheta[i] = flux sum_c s_c dK_c/dtheta_i for theta = (beta+,
 * beta-, M_Z, Gamma_Z) at the theta of cfg, r = bin_weight as in
 * tp_binned_adjoint. Either output may be NULL. */
int tp_grad(tp_ctx *ctx, const tp_config *cfg, int rng_kind, uint64_t seed,
            uint64_t first_batch, uint64_t n_batches, int precision,
            const tp_binning *bins, const double *bin_weight,
            double dlnl_dtheta[4], double dsigma_dtheta[4]);

/* K_c(theta) and dK_c/d(beta+, beta-, M_Z, Gamma_Z) (dk[4 c + i], forward-
 * mode dual numbers) at the theta of cfg, and the incident flux 1/(2 s)
 * (src/resacc.rs:178) that turns sums of w into cross sections (pb). */
int tp_coupling_factors(const tp_config *cfg, double k[5], double dk[20],
                        double *flux);

/* ---- measurement (no counterpart in the reference, which only measures
 * its wall-clock time, src/main.rs:85,138) ------------------------------
 * tp_profile(ctx, 1) starts recording a CUDA event pair around every kernel
 * the context launches; tp_profile_read() waits for them and returns the
 * summed device time (ms) and launch count of the event kernels and of the
 * stream-seeding kernels, then clears the record. tp_profile(ctx, 0) stops.
 * tp_probe_fp64 measures this device's FP64 rates: out[0] = DFMA
 * throughput in flop/s (an FMA counts 2), out[1..4] = the cost of one
 * log, sincos, sqrt and division in DFMA-equivalents. */
int tp_profile(tp_ctx *ctx, int enable);
int tp_profile_read(tp_ctx *ctx, double *event_ms, uint64_t *event_launches,
                    double *seed_ms, uint64_t *seed_launches);
int tp_probe_fp64(tp_ctx *ctx, double out[5]);
/* tp_probe_fp32 measures this device's FP32 rates: out[0] = FFMA throughput
 * in flop/s (an FMA counts 2), out[1] = special-function (MUFU log2)
 * operations per second. */
int tp_probe_fp32(tp_ctx *ctx, double out[2]);

/* Number of events the FP32-mixed path handed to its FP64 recheck (events
 * whose cut decision lay within the FP32 error bound) since the context was
 * created or the counter last reset (reset != 0 clears it after reading).
 * The reference has no mixed-precision path. */
int tp_recheck_count(tp_ctx *ctx, uint64_t *count, int reset);

/* The precision form's error, batch by batch: runs batches [first_batch,
 * first_batch + n_batches) of the stream in FP32-mixed and in FP64 (the same
 * events) and writes err_vs_fp64[i] = the largest relative difference of
 * batch i's sums (spm2[5], vars[5], sigma, variance; the mixed terms on the
 * scale of the A sum), or -1 where the selected counts differ. Either run's
 * sums may be returned through the optional fp32 / fp64 arrays (NULL to
 * skip). No counterpart in the reference, which has no mixed-precision
 * path. */
int tp_fp32_error(tp_ctx *ctx, const tp_config *cfg, int rng_kind,
                  uint64_t seed, uint64_t first_batch, uint64_t n_batches,
                  double *err_vs_fp64, tp_batch_soa *fp32, tp_batch_soa *fp64);

/* ---- host-side jump-ahead (no GPU) ----------------------------------------
 * State of a stream after `draws` draws, computed by polynomial jump-ahead:
 * checkpoint/resume and sharding need no stepping. xoshiro: seed_from_u64
 * (src/random/standard.rs:21-25), then `jumps128` RandomGenerator::jump()
 * calls (standard.rs:53-55), then `draws` draws. ranf: seeded_new
 * (src/random/ranf.rs:36-66) then `draws` draws: slots 1..55 and the
 * remaining draws of the current block (`index`). Returns
 * TP_ERR_UNSUPPORTED when the ranf seed leaves its state outside [0, 1e9). */
int tp_xoshiro_state_at(uint64_t seed, uint64_t jumps128, uint64_t draws,
                        uint64_t state[4]);
int tp_ranf_state_at(int32_t seed, uint64_t draws, int32_t slots[55],
                     int32_t *index);

/* ---- allocation-free batches -----------------------------------------------
 * No counterpart in the reference. For callers that must not allocate GPU
 * memory when they want events: real-time or embedded hosts that plan all
 * GPU memory at start-up, programs whose GPU memory belongs to another
 * allocator (a framework's caching pool) that this library must not
 * bypass. Same work as tp_run_batches_async for the xoshiro256+ stream:
 * rng_kind = TP_RNG_XOSHIRO256P, optionally OR-ed with
 * TP_MODE_JUMP_PER_BATCH and/or TP_MODE_NO_PHOTON_SORTING (other flags,
 * TP_MODE_FASTER_EVGEN included, give TP_ERR_INVALID); FP64 or
 * FP32-mixed; on the CURRENT CUDA device and the given stream (a
 * cudaStream_t; NULL is the default stream), writing the caller's DEVICE
 * arrays `out`. No context, no cudaMalloc/cudaFree: the working memory (the
 * start state of each batch and the jump-ahead tables) lives in fixed
 * arrays of the library, 140 KiB per GPU that loads the library, held until
 * the process exits.
 *  - at most TP_NOALLOC_MAX_BATCHES batches per call; larger ranges fail
 *    with TP_ERR_INVALID: split them into several calls. Batches at or past
 *    ceil(num_events / TP_BATCH_SIZE) hold no events and come back with
 *    zero sums, as in tp_run_batches;
 *  - the first call on a device sets that device up (looks up the arrays'
 *    addresses, uploads the tables with a synchronous copy): make that
 *    first call before any stream capture. After a cudaDeviceReset the next
 *    call sets the device up again (it checks the context's ID);
 *  - every call shares the same working memory, so calls that overlap on
 *    the GPU (other streams, other host threads) race; order them on one
 *    stream or synchronise between them. Nothing in it needs clearing: each
 *    call writes every entry it reads;
 *  - errors: a negative TP_ERR_*, message in tp_last_error(NULL). */
#define TP_NOALLOC_MAX_BATCHES 4096
int tp_run_batches_noalloc(const tp_config *cfg, int rng_kind, uint64_t seed,
                           uint64_t first_batch, uint64_t n_batches,
                           int precision, tp_batch_soa *out, void *stream);

/* ========================================================================
 * Host side kept from the reference (no GPU needed)
 * ======================================================================== */

/* Parses a `valeurs` file: the first whitespace-separated token of every
 * non-blank line, 18 items (Configuration::load, src/config.rs:57-128),
 * and applies its checks (num_events > 0, plot and impr false). If `echo`
 * is non-NULL, the configuration echo of src/config.rs:131-155 is written
 * there (NUL-terminated, truncated to echo_len). */
int tp_config_load(const char *path, tp_config *out, char *echo,
                   size_t echo_len);

/* The two values the reference computes once per run on the host:
 * EventGenerator::event_weight (src/evgen.rs:40-77) and the couplings
 * (src/coupling.rs:23-33). */
int tp_event_weight(double e_total, double *weight);

/* Merges n_batches per-batch accumulators in batch order
 * (ResultsAccumulator::merge, src/resacc.rs:133-139) and finalises them
 * (ResultsAccumulator::finalize, src/resacc.rs:142-223). */
int tp_merge_finalize(const tp_config *cfg, const tp_batch_soa *batches,
                      uint64_t n_batches, tp_final_results *res);

/* res.data text (src/output.rs:62-142) into `buf` (NUL-terminated,
 * truncated). Returns the full length needed, or a negative TP_ERR_* code. */
int tp_format_res_data(const tp_config *cfg, const tp_final_results *res,
                       char *buf, size_t buf_len);

/* Writes res.data exactly as src/output.rs:62-142 does. */
int tp_write_res_data(const tp_config *cfg, const tp_final_results *res,
                      const char *path);

/* The two other files of a run (src/output.rs:35-60, 144-173): res.times
 * (UTC timestamp and elapsed seconds) and one appended record in pil.mc.
 * `timestamp` is the "dd-Mon-yy HH:MM:SS" stamp of the run's end; NULL
 * takes the current UTC time. */
int tp_write_res_times(const tp_config *cfg, double elapsed_seconds,
                       const char *timestamp, const char *path);
int tp_append_pil_mc(const tp_config *cfg, const tp_final_results *res,
                     const char *timestamp, const char *path);

/* Formats the physics printout of FinalResults::eric and ::fawzi
 * (src/resfin.rs:66-194) into `buf` (NUL-terminated, truncated). Returns
 * the full length needed, or a negative TP_ERR_* code. */
int tp_format_report(const tp_config *cfg, const tp_final_results *res,
                     char *buf, size_t buf_len);

#ifdef __cplusplus
}
#endif

#endif /* TP_GPU_H */
