// tp_internal.h — types shared by the kernels (tp_kernels.cu) and the host
// code (tp_host.cpp, tp_capi.cpp). Not part of the public ABI.
#ifndef TP_INTERNAL_H
#define TP_INTERNAL_H

#include <cstddef>
#include <cstdint>

#include "../../include/tp_gpu.h"

namespace tp {

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kMinPositive = 2.2250738585072014e-308;  // f64::MIN_POSITIVE
constexpr int kBatch = TP_BATCH_SIZE;
constexpr int kDrawsPerEvent = 12;  // default evgen: 3 photons x 4 draws
constexpr uint64_t kDrawsPerBatch = (uint64_t)kDrawsPerEvent * kBatch;
// blocks of 55 draws a warp may have to jump within one batch:
// (54 + 12e4) / 55 + 1
constexpr int kRanfBlocksInBatch = (54 + (int)kDrawsPerBatch) / 55 + 1;

// Per-run constants of the event path, computed once on the host.
struct EvConst {
  double e_total;  // sqrt(s)
  double half;     // e_total / 2: E of both beams, p_x of the positron
  double em_x;     // -e_total / 2: p_x of the electron (src/evgen.rs:66-69)
  double acut, bcut, emin, sincut;
  // Couplings::new (src/coupling.rs:23-33)
  double g_a, g_bp, g_bm;
  // ResultsAccumulator::sigma_contribs (src/resacc.rs:88-100)
  double sc[5];
  // Spinor constants of the two beams (src/spinor.rs:37-52): xx = sqrt(E+Z)
  // and fx = p_x / xx for e- and e+, s(e-, e+) and the amplitude prefactors
  // c1 = -RAC8 s(e-,e+), c2 = -RAC8 t(e-,e+).
  double xx_in, fx_em, fx_ep, s01, c1, c2;
  // factors turning the kernels' unscaled helicity sums into the
  // reference's m2_sums: (g_a c1)^2, (g_bp c1)^2, (g_bm c1)^2,
  // -2 g_a g_bp c1^2 (real and imaginary mixed parts)
  double sc_raw[4];
  // FP32 copies for the mixed-precision path
  float f_e_total, f_half, f_em_x, f_acut, f_bcut, f_emin, f_sincut;
  float f_acut_half;  // acut * half rounded once (the beam cut's threshold per unit of E)
  float f_xx_in, f_fx_em, f_fx_ep, f_c1, f_c2;
  // The FP32 helicity sums are computed from momenta scaled by 1 / lambda,
  // lambda = 2^ceil(log2(sqrt(s) / 2)) (exact), and come out as raw_c /
  // hat_scale[c] (each sum is homogeneous in the momenta); f_sc_raw, f_K
  // include hat_scale, f_raw_to_hat = 1 / hat_scale (the direct formulas'
  // sums into the scaled ones)
  float f_inv_lambda;
  float f_sc_raw[5];
  float f_raw_to_hat[5], f_raw_to_hat_lo[5];
  double hat_scale[5];
  // the FP32 batch sums are taken on the scaled sums and multiplied by
  // sc_raw_hat (and its square) in FP64 at the batch reduction, which also
  // forms sigma from them with K hat_scale in FP64; only the squared event
  // weight (the variance) uses K's FP32 rounding f_K
  double sc_raw_hat[5];
  float f_sc[5];
  // per-event weight w = sum_c raw_c * K_c (K = sc_raw * sc, see above)
  double K[5];
  float f_K[5];
  int flags;  // TP_MODE_* bits
};

// Per-batch outputs in SoA layout: element [c * stride + i]
struct BatchOut {
  uint64_t* selected;
  double* spm2;
  double* vars;
  double* sigma;
  double* variance;
  uint64_t stride;
};

struct KParams {
  EvConst k;
  uint64_t first_batch;  // absolute index of the launch's first batch
  uint64_t n_batches;
  uint64_t num_events;   // events of the whole run
  int ept;               // xoshiro: events per thread
  int occupancy;         // xoshiro event kernels: minimum CTAs per SM (2 or 3)
  int precision;
  const void* batch_state;     // xoshiro: 4 x u64 per batch; ranf: 56 x i32
  const uint64_t* thread_poly; // xoshiro: x^(12 ept j) mod P, 4 words per j
  const uint64_t* jump_tab;    // xoshiro: the same jumps as tables (kJumpTabWords per j), or null
  const uint32_t* ranf_table;  // ranf: x^(55 2^k) mod P, 55 coefficients per k
  const uint32_t* ranf_blocks; // ranf: x^(55 D) mod P for D < kRanfBlocksInBatch
  BatchOut out;
  unsigned int* err;     // device error word (0 = fine)
  unsigned long long* recheck_count;  // FP32-mixed: events decided by the FP64 recheck
  // binned observables: x = E of the most energetic photon, y = cosine of
  // its angle to the electron beam; bin = ix * ny + iy
  int nx, ny;
  double x_lo, x_inv_w, y_lo, y_inv_w;
  float f_x_lo, f_x_inv_w, f_y_lo, f_y_inv_w;  // the same, for the FP32-mixed kernels
  const double* bin_weight;  // adjoint: d lnL / d mu_b per bin
  double* hist;              // binned forward: [nx * ny][8] accumulators
  double* adj;               // adjoint: [n_batches][10] per-batch sums
};

// Batched form: many parameter points in one persistent launch. Work unit
// u = one 10k batch of one point; units are numbered point by point.
struct PointsParams {
  int kind;                         // TP_RNG_XOSHIRO256P or TP_RNG_RANF
  const EvConst* points;            // [n_points]
  const uint64_t* point_events;     // [n_points] events of each point's run
  const uint64_t* point_unit0;      // [n_points] first unit of each point
  const uint64_t* point_start;      // xoshiro: [n_points][4] state at draw 0
  const int32_t* point_window;      // ranf: [n_points][110] blocks 0 and 1 of the point's stream
  const uint32_t* unit_point;       // [n_units]
  const uint64_t* batch_table;      // xoshiro: 64 x 4: x^(12e4 * 2^k)
  const uint64_t* thread_poly;      // xoshiro: x^(12 ept j)
  const uint64_t* jump_tab;         // xoshiro: the same as tables, or null
  const uint32_t* ranf_table;       // ranf: x^(55 2^k) mod P
  const uint32_t* ranf_blocks;      // ranf: x^(55 D) mod P for D < kRanfBlocksInBatch
  void* unit_state;                 // [n_units] scratch: batch start states (xoshiro 4 x u64, ranf 56 x i32)
  unsigned long long* counter;      // work-queue head, 0 at launch
  unsigned long long* recheck_count;
  BatchOut out;                     // stride n_units
  uint64_t n_units;
  int ept;
  int precision;
  int occupancy;  // FP32-mixed: kernel variant, minimum CTAs per SM (2 or 3)
};

// faster-evgen (src/evgen.rs:143-173, 221-249): an event takes 15 draws plus
// 2 per rejected point, so event boundaries are found before the physics.
// A stream's draw positions are cut into chunks of kFeChunk; an event
// belongs to the chunk of its first draw. A chunk's CTA (two warps)
// computes the accept bits of kFeSpan positions (the chunk and a margin for
// the events that run past its end: 2048 draws, an event of a thousand
// re-rolls), 544 per xoshiro lane.
constexpr uint32_t kFeChunk = 32768;
constexpr uint32_t kFeSpan = 34816;
constexpr int kFeThreads = 64;  // threads of the chunk kernels
constexpr uint32_t kFeLaneSpan = kFeSpan / kFeThreads;
constexpr int kFeEntries = 32;             // entry offsets per chunk map
constexpr uint32_t kFeMapError = 0xffffffffu;
constexpr int kFeMaxStarts = 128;          // thread starts recorded per chunk
constexpr int kFeMaxTries = 2048;          // re-rolls per point: an event stops after 3 kFeMaxTries
// error bits set by the faster-evgen kernels
constexpr unsigned kFeErrSpan = 0x10u;     // an event ran past the chunk's span
constexpr unsigned kFeErrStarts = 0x20u;   // too many thread starts in a chunk
constexpr unsigned kFeErrTries = 0x40u;    // an event re-rolled its points 3 kFeMaxTries times

// One chunk of a stream: for the map pass, lane l maps entry offset
// entry + l; for the starts pass, entry is the offset of the chunk's first
// event and first_event its index within the stream.
struct FeChunk {
  uint64_t stream;  // one-stream runs: 0; per-batch streams: the batch
  uint64_t chunk;   // positions [chunk * kFeChunk, ...) of the stream
  uint64_t first_event;
  uint32_t entry;
  uint32_t events;  // starts pass: events that start in the chunk (from the composition)
};

struct FeParams {
  int kind;                      // TP_RNG_RANF or TP_RNG_XOSHIRO256P
  int jpb;                       // per-batch streams (TP_MODE_JUMP_PER_BATCH)
  uint64_t xo_start[4];          // xoshiro state at draw 0 of the seed
  int32_t ranf_seed;
  const int32_t* ranf_window;    // one-stream ranf: blocks 0 and 1 of the stream
  const uint32_t* ranf_table;    // x^(55 2^k) mod P
  const uint64_t* xo_stream;     // x^(2^128 2^k): per-batch stream starts
  const uint64_t* xo_chunk;      // x^(kFeChunk 2^k)
  const uint64_t* xo_lane_tab;   // x^(kFeLaneSpan l), l < kFeThreads, as jump tables (kJumpTabWords each)
  const FeChunk* chunks;
  uint64_t n_chunks;
  void* chunk_state;             // per chunk: xoshiro 4 x u64; ranf 2 x 56 i32, at the chunk's
                                 // start and at position kFeSpan / 2 (the map pass's two warps)
  uint32_t* map;                 // map pass: [n_chunks][32] exit << 16 | events
  // starts pass: thread t of batch first_batch + i starts event
  // kBatch (first_batch + i) + ept t; its stream state goes to
  // thread_state[i * tpb + t] (xoshiro 4 x u64, ranf 56 x i32)
  uint64_t first_batch, n_batches, num_events;
  int ept, tpb;
  void* thread_state;
  unsigned int* err;
  // one-stream runs: the map pass keeps each chunk's accept bits and
  // sub-span chases (kFeStoreWords words) and its stream checkpoints
  // (xoshiro: kFeCkptWords u64, ranf: kFeRanfCkptInts i32) for the starts
  // pass; chunks >= store_chunks (or a null store) regenerate them
  uint32_t* bits_store;
  uint64_t* ckpt_store;
  uint64_t store_chunks;
};
// The chunk kernels chase each of kFeSubs sub-spans of kFeSub positions
// (one lane each) from kFeLead positions before it; a walk through the
// chunk then jumps over every sub-span whose chase it meets.
constexpr int kFeSubs = 32;
constexpr uint32_t kFeSub = kFeChunk / kFeSubs;  // 1024 positions
constexpr uint32_t kFeLead = 2048;
// bit store words per chunk: bits A and B, the chases' marks and exits,
// the map pass's walks (per sub-span and entry lane: the walk's first
// event start in the sub-span | the events before it << 16) and the entry
// offset of lane 0; 16-byte aligned parts
constexpr uint32_t kFeStoreCanon = 2 * (kFeSpan / 32);
constexpr uint32_t kFeStoreExit = kFeStoreCanon + kFeChunk / 32;
constexpr uint32_t kFeStoreTrace = kFeStoreExit + kFeSubs;
constexpr uint32_t kFeStoreEntry = kFeStoreTrace + kFeSubs * kFeEntries;
constexpr uint32_t kFeStoreWords = kFeStoreEntry + 4;
// xoshiro checkpoints per lane: the states at 544 l + 128 k + 3, k < 5;
// per chunk those of the kFeThreads lanes, then the chunk's start state
constexpr uint32_t kFeCkpts = (kFeLaneSpan / 32 + 3) / 4;
constexpr uint32_t kFeCkptStart = kFeThreads * kFeCkpts * 4;
constexpr uint32_t kFeCkptWords = kFeCkptStart + 4;
// ranf checkpoints per chunk: the block (slots 1..55 at [1..55] of 56
// ints) after every kFeRanfCkptBlocks resets from the block holding the
// chunk's first draw, through the chunk's last block (596 resets)
constexpr uint32_t kFeRanfCkptBlocks = 32;
constexpr uint32_t kFeRanfCkpts = (54 + kFeChunk - 1) / 55 / kFeRanfCkptBlocks + 1;
constexpr uint32_t kFeRanfCkptInts = kFeRanfCkpts * 56;
// ranf: rows kFeRanfStepRow.. of the x^(55 2^k) table hold x^(55 n) for the
// block distances n = 595, 596 between consecutive chunks' first draws and
// n = 316, 317 from a chunk's first draw to its second state (kFeSpan / 2 on)
constexpr int kFeRanfStepRow = 64;
constexpr int kRanfTableRows = kFeRanfStepRow + 4;
static_assert(kFeChunk / 55 == 595 && (kFeSpan / 2) / 55 == 316, "ranf chunk step table");

// per-bin record of the binned forward pass
constexpr int kBinStride = 8;  // raw sums R_0..R_4, events, sum w, sum w^2
constexpr int kMaxBins = 1024;

// Host-side helpers (tp_host.cpp)
int make_ev_const(const tp_config& cfg, int flags, EvConst* k);
double event_weight(double e_total);
int check_config(const tp_config* cfg);

// Kernel launchers (tp_kernels.cu); `stream` is a cudaStream_t
int launch_seed_xoshiro(const uint64_t start[4], const uint64_t* d_table, uint64_t first_batch,
                        uint64_t n_batches, uint64_t* d_out, void* stream);
int launch_seed_ranf(int jump_per_batch, int32_t seed, const int32_t* d_window, const uint32_t* d_table,
                     const uint32_t* d_blocks, uint64_t first_batch, uint64_t n_batches, int32_t* d_out,
                     void* stream);
int launch_events(int rng_kind, const KParams& p, int tpb, void* stream);
int launch_dump(int rng_kind, int precision, const EvConst& k, const uint64_t start[4], const int32_t* d_window,
                int32_t seed, const uint64_t* d_xo_draw_table, const uint64_t* d_xo_jump_table,
                const uint32_t* d_ranf_table, uint64_t first_event, uint64_t n,
                tp_event_dump* d_out, unsigned int* d_err, void* stream);

// message returned by tp_last_error(NULL) on this thread
void set_thread_error(const char* msg);
int launch_probe(int op, int iters, int blocks, int tpb, double* d_sink, void* stream);
int launch_binned(int rng_kind, const KParams& p, int tpb, int grid, void* stream);
int launch_points(const PointsParams& p, int tpb, void* stream);
// Four-Russians tables of a thread's xoshiro jump J(T): for each group g of
// 4 state bits (64 groups) and each value v of the group, the XOR of the
// images J(T) e_i of the group's set bits: 64 x 16 entries of 4 words.
constexpr int kJumpTabWords = 64 * 16 * 4;
int launch_build_jump_tab(const uint64_t* d_poly, int n_threads, uint64_t* d_tab, void* stream);
int points_grid(int precision, int occupancy, int tpb);  // persistent grid size on the current device
int events_wave(int precision, int occupancy, int tpb);  // resident xoshiro event CTAs on the current device
int launch_adjoint(int rng_kind, const KParams& p, int tpb, void* stream);
// faster-evgen passes: chunk start states, chunk maps, thread start states,
// events (batch_state = the thread start states)
int launch_fe_seed(const FeParams& p, void* stream);
int launch_fe_map(const FeParams& p, void* stream);
int launch_fe_starts(const FeParams& p, void* stream);
// one kept chunk's map from an entry offset >= kFeEntries, from the store
int launch_fe_walk_kept(const FeParams& p, uint64_t chunk, uint32_t entry, uint32_t* d_out, void* stream);
int launch_fe_events(int rng_kind, const KParams& p, int tpb, void* stream);

}  // namespace tp

#endif
