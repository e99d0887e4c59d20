// tp_capi.cpp — the C ABI of include/tp_gpu.h around the kernels: context,
// device buffers, jump-ahead tables, batching of launches, error reporting.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "tp_internal.h"
#include "tp_rng.h"

namespace {

using namespace tp;

thread_local std::string g_create_error;

}  // namespace

namespace tp {
void set_thread_error(const char* msg) { g_create_error = msg; }
}  // namespace tp

namespace {

// Batches per launch: bounds the device scratch (batch start states) to
// 64 Ki batches = 14.7 MB (ranf) or 2 MB (xoshiro).
constexpr uint64_t kChunk = 1ull << 16;
constexpr int kTpb = 256;      // threads per CTA (one batch per CTA)
constexpr int kDefaultEpt = 40;  // xoshiro: events per thread (250 x 40)
constexpr int kBinnedEpt = 313;  // binned passes: one warp per batch (measured fastest for both)

struct Tables {
  std::vector<uint64_t> xo_batch, xo_jump, xo_draw;  // 64 x 4 words each
  std::vector<uint64_t> xo_fe_chunk;                  // 64 x 4: x^(kFeChunk 2^k)
  std::vector<uint64_t> xo_fe_lane;                   // kFeThreads x 4: x^(kFeLaneSpan l)
  std::vector<uint32_t> ranf;                         // kRanfTableRows x 55
};

const Tables& host_tables() {
  static Tables t;
  static std::once_flag once;
  std::call_once(once, [] {
    t.xo_batch.resize(256);
    t.xo_jump.resize(256);
    t.xo_draw.resize(256);
    Gf2Poly pb = gf2_xpow(kDrawsPerBatch), pj = gf2_xpow2k(128), pd = gf2_xpow(kDrawsPerEvent);
    for (int k = 0; k < 64; ++k) {
      for (int w = 0; w < 4; ++w) {
        t.xo_batch[4 * k + w] = pb.w[w];
        t.xo_jump[4 * k + w] = pj.w[w];
        t.xo_draw[4 * k + w] = pd.w[w];
      }
      pb = gf2_mulmod(pb, pb);
      pj = gf2_mulmod(pj, pj);
      pd = gf2_mulmod(pd, pd);
    }
    t.xo_fe_chunk.resize(256);
    Gf2Poly pc = gf2_xpow(kFeChunk);
    for (int k = 0; k < 64; ++k) {
      for (int w = 0; w < 4; ++w) t.xo_fe_chunk[4 * k + w] = pc.w[w];
      pc = gf2_mulmod(pc, pc);
    }
    t.xo_fe_lane.resize(4 * kFeThreads);
    const Gf2Poly lane_step = gf2_xpow(kFeLaneSpan);
    Gf2Poly cur{{1, 0, 0, 0}};
    for (int l = 0; l < kFeThreads; ++l) {
      for (int w = 0; w < 4; ++w) t.xo_fe_lane[4 * l + w] = cur.w[w];
      cur = gf2_mulmod(cur, lane_step);
    }
    t.ranf.resize(kRanfTableRows * 55);
    RanfPoly r = ranf_xpow(55);
    for (int k = 0; k < 64; ++k) {
      for (int i = 0; i < 55; ++i) t.ranf[55 * k + i] = r.c[i];
      r = ranf_mulmod(r, r);
    }
    const uint64_t steps[4] = {595, 596, 316, 317};
    for (int k = 0; k < 4; ++k) {
      const RanfPoly s = ranf_xpow(55 * steps[k]);
      for (int i = 0; i < 55; ++i) t.ranf[55 * (kFeRanfStepRow + k) + i] = s.c[i];
    }
  });
  return t;
}

}  // namespace

struct tp_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // per precision (FP64, FP32-mixed): xoshiro events per thread and event
  // kernel variant (min CTAs per SM)
  // [2]: the binned forward and adjoint passes (their own shape: one-warp
  // batches, eight per CTA in the forward pass; not autotuned)
  int ept[3] = {kDefaultEpt, kDefaultEpt, kBinnedEpt};
  int occupancy[2] = {2, 2};
  uint64_t* d_xo_batch = nullptr;
  uint64_t* d_xo_jump = nullptr;
  uint64_t* d_xo_draw = nullptr;
  uint32_t* d_ranf_tab = nullptr;
  uint32_t* d_ranf_blocks = nullptr;  // x^(55 D), D < kRanfBlocksInBatch (built on first ranf run)
  uint64_t* d_thread_poly[3] = {nullptr, nullptr, nullptr};  // per ept slot: x^(12 ept j), j < 256
  uint64_t* d_jump_tab[3] = {nullptr, nullptr, nullptr};     // the same jumps as tables (8 MiB; not slot 2)
  int thread_poly_ept[3] = {0, 0, 0};
  int32_t* d_ranf_window = nullptr;
  int64_t ranf_window_seed = -1;
  void* d_state = nullptr;
  void* d_out = nullptr;
  size_t out_bytes = 0;
  void* d_dump = nullptr;
  size_t dump_bytes = 0;
  unsigned int* d_err = nullptr;
  unsigned long long* d_recheck = nullptr;  // FP32-mixed events settled in FP64
  double* d_hist = nullptr;   // binned forward: kMaxBins x kBinStride
  double* d_binw = nullptr;   // adjoint: bin weights (kMaxBins)
  double* d_adj = nullptr;    // adjoint: per-batch sums, kChunk x 10
  // faster-evgen: jump tables, chunk list, chunk states, chunk maps, thread start states
  uint64_t* d_xo_fe_chunk = nullptr;
  uint64_t* d_xo_fe_lane = nullptr;
  uint64_t* d_fe_lane_tab = nullptr;  // the lane jumps as tables (2 MiB)
  void* d_fe_chunks = nullptr;
  size_t fe_chunks_bytes = 0;
  void* d_fe_cstate = nullptr;
  size_t fe_cstate_bytes = 0;
  void* d_fe_map = nullptr;
  size_t fe_map_bytes = 0;
  void* d_fe_tstate = nullptr;
  size_t fe_tstate_bytes = 0;
  void* d_fe_store = nullptr;  // one-stream runs: accept bits and lane states per chunk
  uint32_t* h_fe_maps = nullptr;  // pinned host copy of a map launch's maps
  size_t h_fe_maps_bytes = 0;
  uint64_t fe_store_cap = 16ull << 30;  // bytes the bit store may take
  size_t fe_store_bytes = 0;
  int sms = 0;
  // batched form (tp_run_points): device buffers and the captured graph
  struct Points {
    void* buf = nullptr;  // points, events, unit0, starts, unit_point, states, outputs, counter
    size_t bytes = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t key[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // n_points, n_units, precision, ept, flags, buffer, variant, kind
  } pts;
  // optional CUDA-event timing of every kernel launch (tp_profile)
  int prof = 0;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_marks;  // (kind, start/end)
  size_t ev_used = 0;

  cudaEvent_t next_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }

  int fail(int code, const std::string& msg) {
    err = msg;
    return code;
  }
  int cuda(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return TP_OK;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return TP_ERR_CUDA;
  }
};

namespace {

int ensure(tp_ctx* c, void** p, size_t* have, size_t need, const char* what) {
  if (*have >= need) return TP_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *have = 0;
  int st = c->cuda(cudaMalloc(p, need), what);
  if (st == TP_OK) *have = need;
  return st;
}

int prec_index(int precision) { return precision == TP_PREC_FP32_MIXED ? 1 : 0; }

// Thread jump polynomials and tables of ept slot `slot` (0 FP64, 1
// FP32-mixed, 2 the binned passes) for its current events per thread.
int ensure_thread_poly(tp_ctx* c, int slot) {
  const int ept = c->ept[slot];
  if (c->thread_poly_ept[slot] == ept) return TP_OK;
  std::vector<uint64_t> h(4 * kTpb);
  const Gf2Poly step = gf2_xpow((uint64_t)kDrawsPerEvent * ept);
  Gf2Poly cur{{1, 0, 0, 0}};
  for (int j = 0; j < kTpb; ++j) {
    for (int w = 0; w < 4; ++w) h[4 * j + w] = cur.w[w];
    cur = gf2_mulmod(cur, step);
  }
  int st = c->cuda(cudaMemcpyAsync(c->d_thread_poly[slot], h.data(), h.size() * 8, cudaMemcpyHostToDevice, c->stream),
                   "upload thread polynomials");
  if (st) return st;
  if (c->d_jump_tab[slot] &&
      launch_build_jump_tab(c->d_thread_poly[slot], kTpb, c->d_jump_tab[slot], c->stream) != TP_OK)
    return c->fail(TP_ERR_CUDA, "building the thread jump tables failed");
  st = c->cuda(cudaStreamSynchronize(c->stream), "upload thread polynomials");
  if (st == TP_OK) c->thread_poly_ept[slot] = ept;
  return st;
}

// x^(55 D) mod P for every jump a warp of a ranf event kernel may make
// within a batch, so that each warp positions its stream with one product
int ensure_ranf_blocks(tp_ctx* c) {
  if (c->d_ranf_blocks) return TP_OK;
  std::vector<uint32_t> h(55 * (size_t)kRanfBlocksInBatch);
  const RanfPoly step = ranf_xpow(55);
  RanfPoly cur = ranf_xpow(0);
  for (int d = 0; d < kRanfBlocksInBatch; ++d) {
    for (int i = 0; i < 55; ++i) h[55 * (size_t)d + i] = cur.c[i];
    cur = ranf_mulmod(cur, step);
  }
  uint32_t* dev = nullptr;
  int st = c->cuda(cudaMalloc(&dev, h.size() * 4), "ranf block table");
  if (!st) st = c->cuda(cudaMemcpy(dev, h.data(), h.size() * 4, cudaMemcpyHostToDevice), "ranf block table");
  if (st) {
    if (dev) cudaFree(dev);
    return st;
  }
  c->d_ranf_blocks = dev;
  return TP_OK;
}

// blocks 0 and 1 of a ranf stream (110 values) for the one-stream mode
int ensure_ranf_window(tp_ctx* c, int32_t seed) {
  if (c->ranf_window_seed == (int64_t)seed) return TP_OK;
  int32_t w[110];
  ranf_seeded(seed, w);
  if (!ranf_canonical(w))
    return c->fail(TP_ERR_UNSUPPORTED, "ranf seed gives a state outside [0, 1e9): no jump-ahead");
  for (int i = 0; i < 55; ++i) w[55 + i] = w[i];
  ranf_reset(w + 55);
  int st = c->cuda(cudaMemcpyAsync(c->d_ranf_window, w, sizeof w, cudaMemcpyHostToDevice, c->stream),
                   "upload ranf window");
  if (st) return st;
  st = c->cuda(cudaStreamSynchronize(c->stream), "upload ranf window");
  if (st == TP_OK) c->ranf_window_seed = seed;
  return st;
}

int check_kind(tp_ctx* c, int rng_kind, bool faster_evgen_ok = false) {
  const int kind = rng_kind & TP_RNG_KIND_MASK;
  if (kind != TP_RNG_RANF && kind != TP_RNG_XOSHIRO256P) return c->fail(TP_ERR_INVALID, "unknown rng kind");
  if (rng_kind & ~(TP_RNG_KIND_MASK | TP_MODE_JUMP_PER_BATCH | TP_MODE_NO_PHOTON_SORTING | TP_MODE_FASTER_EVGEN))
    return c->fail(TP_ERR_INVALID, "unknown mode flag");
  if ((rng_kind & TP_MODE_FASTER_EVGEN) && !faster_evgen_ok)
    return c->fail(TP_ERR_UNSUPPORTED, "TP_MODE_FASTER_EVGEN is served by tp_run_batches and tp_run_batches_async only");
  return TP_OK;
}

int check_seed(tp_ctx* c, int rng_kind, uint64_t seed) {
  if ((rng_kind & TP_RNG_KIND_MASK) == TP_RNG_RANF && seed > 0x7fffffffull)
    return c->fail(TP_ERR_INVALID, "ranf seed must fit in i32");
  return TP_OK;
}

enum class Pass { kBatches, kBinned, kAdjoint };

int run_fe(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch, uint64_t n_batches,
           int precision, const BatchOut& out, cudaStream_t stream);

// Queues the batches on `stream`; `out` holds device pointers (stride n).
// `pass` selects the per-batch accumulators, the binned forward pass or the
// adjoint pass (the latter two take their extra fields from `extra`).
int run_async(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch,
              uint64_t n_batches, int precision, const BatchOut& out, cudaStream_t stream,
              Pass pass = Pass::kBatches, const KParams* extra = nullptr,
              std::vector<double>* adj_host = nullptr) {
  if (check_config(cfg)) return c->fail(TP_ERR_INVALID, "invalid configuration");
  if (int st = check_kind(c, rng_kind, pass == Pass::kBatches)) return st;
  if (int st = check_seed(c, rng_kind, seed)) return st;
  if (n_batches == 0) return TP_OK;
  if (first_batch > (1ull << 46) || n_batches > (1ull << 46))
    return c->fail(TP_ERR_INVALID, "batch range too large");
  if (precision != TP_PREC_FP64 && precision != TP_PREC_FP32_MIXED)
    return c->fail(TP_ERR_INVALID, "unknown precision");
  if (rng_kind & TP_MODE_FASTER_EVGEN)
    return run_fe(c, cfg, rng_kind, seed, first_batch, n_batches, precision, out, stream);
  const int kind = rng_kind & TP_RNG_KIND_MASK;
  const bool jpb = (rng_kind & TP_MODE_JUMP_PER_BATCH) != 0;
  KParams kp{};
  make_ev_const(*cfg, rng_kind & ~TP_RNG_KIND_MASK, &kp.k);
  kp.num_events = cfg->num_events;
  kp.precision = precision;
  kp.err = c->d_err;
  kp.recheck_count = c->d_recheck;
  // the binned forward pass runs several batches per CTA at the tuned
  // shape: its per-CTA shared histogram (up to 96 KB) limits how many CTAs
  // fit on an SM
  const int pi = prec_index(precision);
  const int slot = (pass == Pass::kBinned || pass == Pass::kAdjoint) ? 2 : pi;
  const int ept = c->ept[slot];
  kp.ept = ept;
  kp.occupancy = c->occupancy[pi];
  if (kind == TP_RNG_XOSHIRO256P) {
    if (int st = ensure_thread_poly(c, slot)) return st;
  } else {
    if (int st = ensure_ranf_blocks(c)) return st;
    if (!jpb)
      if (int st = ensure_ranf_window(c, (int32_t)seed)) return st;
  }
  kp.thread_poly = c->d_thread_poly[slot];
  kp.jump_tab = c->d_jump_tab[slot];
  kp.ranf_table = c->d_ranf_tab;
  kp.ranf_blocks = c->d_ranf_blocks;
  if (extra) {
    kp.nx = extra->nx;
    kp.ny = extra->ny;
    kp.x_lo = extra->x_lo;
    kp.x_inv_w = extra->x_inv_w;
    kp.y_lo = extra->y_lo;
    kp.y_inv_w = extra->y_inv_w;
    kp.f_x_lo = extra->f_x_lo;
    kp.f_x_inv_w = extra->f_x_inv_w;
    kp.f_y_lo = extra->f_y_lo;
    kp.f_y_inv_w = extra->f_y_inv_w;
    kp.bin_weight = c->d_binw;
    kp.hist = c->d_hist;
    kp.adj = c->d_adj;
  }
  uint64_t start[4];
  xoshiro_seed(seed, start);
  for (uint64_t c0 = 0; c0 < n_batches; c0 += kChunk) {
    const uint64_t cn = n_batches - c0 < kChunk ? n_batches - c0 : kChunk;
    const uint64_t fb = first_batch + c0;
    int st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (c->prof && (e0 = c->next_event()) && (e1 = c->next_event())) cudaEventRecord(e0, stream);
    if (kind == TP_RNG_XOSHIRO256P)
      st = launch_seed_xoshiro(start, jpb ? c->d_xo_jump : c->d_xo_batch, fb, cn,
                               static_cast<uint64_t*>(c->d_state), stream);
    else
      st = launch_seed_ranf(jpb, (int32_t)seed, c->d_ranf_window, c->d_ranf_tab, c->d_ranf_blocks, fb, cn,
                            static_cast<int32_t*>(c->d_state), stream);
    if (e1) {
      cudaEventRecord(e1, stream);
      c->prof_marks.push_back({0, {e0, e1}});
      e0 = e1 = nullptr;
    }
    if (st) return c->fail(st, std::string("seed launch: ") + cudaGetErrorString(cudaGetLastError()));
    kp.first_batch = fb;
    kp.n_batches = cn;
    kp.batch_state = c->d_state;
    kp.out = out;
    kp.out.selected = out.selected + c0;
    kp.out.spm2 = out.spm2 + c0;
    kp.out.vars = out.vars + c0;
    kp.out.sigma = out.sigma + c0;
    kp.out.variance = out.variance + c0;
    // xoshiro: enough warps for ceil(10000 / ept) threads; ranf: rounds of 256
    const int need = (kBatch + ept - 1) / ept;
    const int tpb = kind == TP_RNG_XOSHIRO256P ? ((need + 31) / 32) * 32 : kTpb;
    if (c->prof && (e0 = c->next_event()) && (e1 = c->next_event())) cudaEventRecord(e0, stream);
    if (pass == Pass::kBatches)
      st = launch_events(rng_kind, kp, tpb, stream);
    else if (pass == Pass::kBinned)
      st = launch_binned(rng_kind, kp, tpb, 0, stream);
    else
      st = launch_adjoint(rng_kind, kp, tpb, stream);
    if (e1) {
      cudaEventRecord(e1, stream);
      c->prof_marks.push_back({1, {e0, e1}});
    }
    if (st) return c->fail(st, std::string("event launch: ") + cudaGetErrorString(cudaGetLastError()));
    if (pass == Pass::kAdjoint && adj_host) {
      const size_t off = adj_host->size();
      adj_host->resize(off + 10 * cn);
      st = c->cuda(cudaMemcpyAsync(adj_host->data() + off, c->d_adj, 10 * cn * sizeof(double),
                                   cudaMemcpyDeviceToHost, stream), "copy adjoint sums");
      if (!st) st = c->cuda(cudaStreamSynchronize(stream), "adjoint");
      if (st) return st;
    }
  }
  return TP_OK;
}

// ---------------------------------------------------------------------------
// faster-evgen (TP_MODE_FASTER_EVGEN). The draws per event vary, so every
// event's first draw is found before the physics:
//  1. map pass: per chunk of kFeChunk draw positions, for 32 entry offsets,
//     the offset where the chunk's last event ends and the chunk's event
//     count (k_fe_map, one CTA per chunk: the accept bits, the sub-span
//     chases and a walk per entry offset);
//  2. on the host, the maps composed along each stream from draw 0: the
//     first event and its offset in every chunk;
//  3. starts pass: per chunk, the stream state at each thread's first event
//     (k_fe_starts);
//  4. the event kernel, one CTA per batch (k_fe_events_fp64).
// One stream (events numbered through the run) or one per batch
// (TP_MODE_JUMP_PER_BATCH: events numbered within the batch).
// ---------------------------------------------------------------------------
constexpr uint64_t kFeMapLaunch = 1u << 19;  // chunks per map launch (~1e9 events)
// batches per starts + events launch: bounds the thread start states to
// 134 MB (xoshiro, 32 B per thread) and 235 MB (ranf, 224 B per thread)
constexpr uint64_t kFePieceXo = 16384, kFePieceRanf = 4096;

struct FeStream {
  uint64_t id = 0;       // 0, or the batch for per-batch streams
  uint64_t target = 0;   // events whose chunk must be known
  uint64_t next_chunk = 0;
  uint64_t events = 0;   // events starting before chunk next_chunk
  uint32_t entry = 0;    // offset of chunk next_chunk's first event
  std::vector<FeChunk> chunks;  // composed chunks (entry, first_event)
  bool done() const { return events >= target; }
};

// Uploads `descs`, seeds their chunk states and runs the map pass (maps:
// where the maps are copied back; pinned: into the context's pinned buffer
// instead, *pinned pointing at them) or the starts pass on them.
int fe_launch(tp_ctx* c, FeParams fp, const std::vector<FeChunk>& descs, bool map_pass, cudaStream_t stream,
              std::vector<uint32_t>* maps, const uint32_t** pinned = nullptr) {
  const size_t n = descs.size();
  if (n == 0) return TP_OK;
  if (int st = ensure(c, &c->d_fe_chunks, &c->fe_chunks_bytes, n * sizeof(FeChunk), "faster-evgen chunks")) return st;
  if (int st = ensure(c, &c->d_fe_cstate, &c->fe_cstate_bytes, n * 112 * sizeof(int32_t), "faster-evgen chunk states"))
    return st;
  if (map_pass)
    if (int st = ensure(c, &c->d_fe_map, &c->fe_map_bytes, n * kFeEntries * sizeof(uint32_t), "faster-evgen maps"))
      return st;
  int st = c->cuda(cudaMemcpyAsync(c->d_fe_chunks, descs.data(), n * sizeof(FeChunk), cudaMemcpyHostToDevice, stream),
                   "upload faster-evgen chunks");
  if (st) return st;
  fp.chunks = static_cast<const FeChunk*>(c->d_fe_chunks);
  fp.n_chunks = n;
  fp.chunk_state = c->d_fe_cstate;
  fp.map = static_cast<uint32_t*>(c->d_fe_map);
  // the starts pass of one-stream chunks in the bit store steps from the
  // checkpoints the map pass kept there: no seeding
  bool seed = true;
  if (!map_pass && fp.bits_store && !fp.jpb) {
    seed = false;
    for (const FeChunk& d : descs) seed |= d.chunk >= fp.store_chunks;
  }
  if (seed && launch_fe_seed(fp, stream) != TP_OK)
    return c->fail(TP_ERR_CUDA, std::string("faster-evgen seed launch: ") + cudaGetErrorString(cudaGetLastError()));
  const int lst = map_pass ? launch_fe_map(fp, stream) : launch_fe_starts(fp, stream);
  if (lst != TP_OK)
    return c->fail(TP_ERR_CUDA, std::string("faster-evgen chunk launch: ") + cudaGetErrorString(cudaGetLastError()));
  if (!map_pass) return TP_OK;
  const size_t bytes = n * kFeEntries * sizeof(uint32_t);
  uint32_t* dst = nullptr;
  if (pinned) {
    if (c->h_fe_maps_bytes < bytes) {
      if (c->h_fe_maps) cudaFreeHost(c->h_fe_maps);
      c->h_fe_maps = nullptr;
      c->h_fe_maps_bytes = 0;
      if (int e = c->cuda(cudaMallocHost((void**)&c->h_fe_maps, bytes), "faster-evgen map buffer")) return e;
      c->h_fe_maps_bytes = bytes;
    }
    dst = c->h_fe_maps;
    *pinned = dst;
  } else {
    maps->resize(n * kFeEntries);
    dst = maps->data();
  }
  st = c->cuda(cudaMemcpyAsync(dst, c->d_fe_map, bytes, cudaMemcpyDeviceToHost, stream), "copy faster-evgen maps");
  if (!st) st = c->cuda(cudaStreamSynchronize(stream), "faster-evgen map pass");
  return st;
}

// Steps 1-2 for `streams`: composes chunks until each stream's target.
int fe_compose(tp_ctx* c, const FeParams& fp, std::vector<FeStream>& streams, cudaStream_t stream) {
  std::vector<FeChunk> descs;
  std::vector<uint32_t> one;
  const uint32_t* maps = nullptr;  // the launch's maps, in the pinned buffer
  for (;;) {
    descs.clear();
    for (FeStream& s : streams) {
      if (s.done()) continue;
      // ~16.64 (xoshiro) or ~17.9 (ranf, block skips) draws per event; a
      // short guess maps the rest in the next round
      const double draws = fp.kind == TP_RNG_RANF ? 18.2 : 16.7;
      const uint64_t need = (uint64_t)((double)(s.target - s.events) * draws / kFeChunk) + 2;
      if (streams.size() == 1) {  // one stream: room for the round's chunks at once, and a margin
        const size_t round = (size_t)(need < kFeMapLaunch ? need : kFeMapLaunch);
        descs.reserve(round);
        s.chunks.reserve(s.chunks.size() + round + round / 32 + 64);
      }
      for (uint64_t k = 0; k < need && descs.size() < kFeMapLaunch; ++k)
        descs.push_back(FeChunk{s.id, s.next_chunk + k, 0, 0, 0});
      if (descs.size() >= kFeMapLaunch) break;
    }
    if (descs.empty()) return TP_OK;
    if (int st = fe_launch(c, fp, descs, true, stream, nullptr, &maps)) return st;
    size_t d = 0;
    for (FeStream& s : streams) {
      while (d < descs.size() && descs[d].stream == s.id && descs[d].chunk == s.next_chunk && !s.done()) {
        uint32_t m;
        if (s.entry < (uint32_t)kFeEntries) {
          m = maps[d * kFeEntries + s.entry];
        } else if (fp.bits_store && !fp.jpb && s.next_chunk < fp.store_chunks) {
          // entered past the 32 mapped offsets, a kept chunk: walk from its
          // offset over what the map pass stored (the starts pass then walks
          // this chunk itself)
          uint32_t* d_out = static_cast<uint32_t*>(c->d_fe_map);
          int st = launch_fe_walk_kept(fp, s.next_chunk, s.entry, d_out, stream);
          if (st)
            return c->fail(TP_ERR_CUDA,
                           std::string("faster-evgen walk launch: ") + cudaGetErrorString(cudaGetLastError()));
          st = c->cuda(cudaMemcpyAsync(&m, d_out, sizeof m, cudaMemcpyDeviceToHost, stream), "faster-evgen walk");
          if (!st) st = c->cuda(cudaStreamSynchronize(stream), "faster-evgen walk");
          if (st) return st;
        } else {  // entered past the 32 mapped offsets: map that offset alone
          std::vector<FeChunk> single{FeChunk{s.id, s.next_chunk, 0, s.entry, 0}};
          if (int st = fe_launch(c, fp, single, true, stream, &one)) return st;
          m = one[0];
        }
        if (m == kFeMapError)
          return c->fail(TP_ERR_DEVICE, "faster-evgen: an event runs past its chunk's accept bits");
        s.chunks.push_back(FeChunk{s.id, s.next_chunk, s.events, s.entry, m & 0xffffu});
        s.events += m & 0xffffu;
        s.entry = m >> 16;
        ++s.next_chunk;
        ++d;
      }
      while (d < descs.size() && descs[d].stream == s.id) ++d;  // maps past the target
    }
  }
}

int run_fe(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch, uint64_t n_batches,
           int precision, const BatchOut& out, cudaStream_t stream) {
  const int kind = rng_kind & TP_RNG_KIND_MASK;
  const bool jpb = (rng_kind & TP_MODE_JUMP_PER_BATCH) != 0;
  const uint64_t n_total = cfg->num_events;
  FeParams fp{};
  fp.kind = kind;
  fp.jpb = jpb;
  fp.err = c->d_err;
  fp.ept = c->ept[0];  // the FP64 shape, for both precisions (the thread starts depend on it)
  const int tpb = (((kBatch + fp.ept - 1) / fp.ept) + 31) / 32 * 32;
  fp.tpb = tpb;
  fp.num_events = n_total;
  if (kind == TP_RNG_XOSHIRO256P) {
    xoshiro_seed(seed, fp.xo_start);
  } else {
    fp.ranf_seed = (int32_t)seed;
    if (!jpb)
      if (int st = ensure_ranf_window(c, (int32_t)seed)) return st;
  }
  fp.ranf_window = c->d_ranf_window;
  fp.ranf_table = c->d_ranf_tab;
  fp.xo_stream = c->d_xo_jump;
  fp.xo_chunk = c->d_xo_fe_chunk;
  fp.xo_lane_tab = c->d_fe_lane_tab;
  KParams kp{};
  make_ev_const(*cfg, rng_kind & ~TP_RNG_KIND_MASK, &kp.k);
  kp.num_events = n_total;
  kp.precision = precision;
  kp.err = c->d_err;
  kp.recheck_count = c->d_recheck;
  kp.ept = fp.ept;
  const size_t state_bytes = kind == TP_RNG_RANF ? 56 * sizeof(int32_t) : 4 * sizeof(uint64_t);
  const uint64_t b_end = first_batch + n_batches;
  // one stream: compose once through the last event of the range
  std::vector<FeStream> one(1);
  if (!jpb) {
    // batches past the run are empty: their event kernel CTAs store zeros
    const uint64_t e_end = b_end * (uint64_t)kBatch < n_total ? b_end * (uint64_t)kBatch : n_total;
    one[0].target = first_batch * (uint64_t)kBatch < n_total ? e_end : 0;
    // the map pass keeps every chunk's accept bits, chases, walks and
    // stream checkpoints for the starts pass when they fit in the context's
    // store cap (xoshiro 15.7 GB and ranf 12.3 GB per 1e9 events)
    const uint64_t chunks = (uint64_t)((double)one[0].target * 18.5 / kFeChunk) + 64;
    const size_t ckpt_bytes =
        kind == TP_RNG_XOSHIRO256P ? kFeCkptWords * sizeof(uint64_t) : kFeRanfCkptInts * sizeof(int32_t);
    const size_t per_chunk = kFeStoreWords * sizeof(uint32_t) + ckpt_bytes;
    if (one[0].target > 0 && (double)chunks * per_chunk <= (double)c->fe_store_cap) {
      if (int st = ensure(c, &c->d_fe_store, &c->fe_store_bytes, chunks * per_chunk, "faster-evgen bit store"))
        return st;
      fp.bits_store = static_cast<uint32_t*>(c->d_fe_store);
      fp.ckpt_store =
          reinterpret_cast<uint64_t*>(static_cast<char*>(c->d_fe_store) + chunks * kFeStoreWords * sizeof(uint32_t));
      fp.store_chunks = chunks;
    }
    if (int st = fe_compose(c, fp, one, stream)) return st;
  }
  const uint64_t piece = kind == TP_RNG_RANF ? kFePieceRanf : kFePieceXo;
  size_t kpos = 0;  // one stream: the first composed chunk that ends past the piece's first event
  for (uint64_t p0 = first_batch; p0 < b_end; p0 += piece) {
    const uint64_t pn = b_end - p0 < piece ? b_end - p0 : piece;
    std::vector<FeChunk> descs;
    if (!jpb) {
      // the chunks holding events [lo, hi), in stream order (their first
      // events ascend, and so do the pieces)
      const uint64_t lo = p0 * (uint64_t)kBatch;
      const uint64_t hi = (p0 + pn) * (uint64_t)kBatch;
      const std::vector<FeChunk>& ch = one[0].chunks;
      auto end_of = [&](size_t k) { return k + 1 < ch.size() ? ch[k + 1].first_event : one[0].events; };
      while (kpos < ch.size() && end_of(kpos) <= lo) ++kpos;
      for (size_t k = kpos; k < ch.size() && ch[k].first_event < hi; ++k)
        if (end_of(k) > ch[k].first_event) descs.push_back(ch[k]);
    } else {
      std::vector<FeStream> streams(pn);
      for (uint64_t i = 0; i < pn; ++i) {
        streams[i].id = p0 + i;
        const uint64_t lo = (p0 + i) * (uint64_t)kBatch;
        streams[i].target = lo >= n_total ? 0 : (n_total - lo < (uint64_t)kBatch ? n_total - lo : kBatch);
      }
      if (int st = fe_compose(c, fp, streams, stream)) return st;
      for (const FeStream& s : streams) descs.insert(descs.end(), s.chunks.begin(), s.chunks.end());
    }
    if (int st = ensure(c, &c->d_fe_tstate, &c->fe_tstate_bytes, (size_t)pn * tpb * state_bytes,
                        "faster-evgen thread states"))
      return st;
    FeParams sp = fp;
    sp.first_batch = p0;
    sp.n_batches = pn;
    sp.thread_state = c->d_fe_tstate;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (c->prof && (e0 = c->next_event()) && (e1 = c->next_event())) cudaEventRecord(e0, stream);
    if (int st = fe_launch(c, sp, descs, false, stream, nullptr)) return st;
    if (e1) {
      cudaEventRecord(e1, stream);
      c->prof_marks.push_back({0, {e0, e1}});
      e0 = e1 = nullptr;
    }
    const uint64_t off = p0 - first_batch;
    kp.first_batch = p0;
    kp.n_batches = pn;
    kp.batch_state = c->d_fe_tstate;
    kp.out = out;
    kp.out.selected = out.selected + off;
    kp.out.spm2 = out.spm2 + off;
    kp.out.vars = out.vars + off;
    kp.out.sigma = out.sigma + off;
    kp.out.variance = out.variance + off;
    if (c->prof && (e0 = c->next_event()) && (e1 = c->next_event())) cudaEventRecord(e0, stream);
    const int st = launch_fe_events(rng_kind, kp, tpb, stream);
    if (e1) {
      cudaEventRecord(e1, stream);
      c->prof_marks.push_back({1, {e0, e1}});
    }
    if (st) return c->fail(st, std::string("faster-evgen event launch: ") + cudaGetErrorString(cudaGetLastError()));
  }
  return TP_OK;
}

int binning_params(tp_ctx* c, const tp_config* cfg, const tp_binning* bins, KParams* kp) {
  if (!bins || bins->n_emax < 1 || bins->n_cos < 1 || (int64_t)bins->n_emax * bins->n_cos > kMaxBins)
    return c->fail(TP_ERR_INVALID, "binning: 1 <= n_emax * n_cos <= 1024");
  double xl = bins->emax_lo, xh = bins->emax_hi, yl = bins->cos_lo, yh = bins->cos_hi;
  if (xl == 0.0 && xh == 0.0) {
    xl = cfg->e_total / 3.0;
    xh = cfg->e_total / 2.0;
  }
  if (yl == 0.0 && yh == 0.0) {
    yl = -cfg->beam_photons_cut;
    yh = cfg->beam_photons_cut;
  }
  if (!(xh > xl) || !(yh > yl)) return c->fail(TP_ERR_INVALID, "binning: empty range");
  kp->nx = bins->n_emax;
  kp->ny = bins->n_cos;
  kp->x_lo = xl;
  kp->x_inv_w = bins->n_emax / (xh - xl);
  kp->y_lo = yl;
  kp->y_inv_w = bins->n_cos / (yh - yl);
  kp->f_x_lo = (float)kp->x_lo;
  kp->f_x_inv_w = (float)kp->x_inv_w;
  kp->f_y_lo = (float)kp->y_lo;
  kp->f_y_inv_w = (float)kp->y_inv_w;
  return TP_OK;
}

}  // namespace

extern "C" {

tp_ctx* tp_create(int device, int* status) {
  auto failc = [&](int code, const std::string& msg) -> tp_ctx* {
    g_create_error = msg;
    if (status) *status = code;
    return nullptr;
  };
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return failc(TP_ERR_NO_DEVICE, "no CUDA device");
  if (device < 0 || device >= n) return failc(TP_ERR_NO_DEVICE, "device index out of range");
  if (cudaSetDevice(device) != cudaSuccess) return failc(TP_ERR_NO_DEVICE, "cudaSetDevice failed");
  tp_ctx* c = new tp_ctx;
  c->device = device;
  const Tables& t = host_tables();
  int st = c->cuda(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "stream");
  size_t dummy = 0;
  void* p;
  auto alloc = [&](void** dst, size_t bytes, const char* what) {
    if (st) return;
    st = c->cuda(cudaMalloc(dst, bytes), what);
  };
  alloc((void**)&c->d_xo_batch, 256 * 8, "tables");
  alloc((void**)&c->d_xo_jump, 256 * 8, "tables");
  alloc((void**)&c->d_xo_draw, 256 * 8, "tables");
  alloc((void**)&c->d_ranf_tab, kRanfTableRows * 55 * 4, "tables");
  // the binned passes (slot 2) jump by polynomial: no table
  for (int k = 0; k < 3; ++k) alloc((void**)&c->d_thread_poly[k], kTpb * 32, "tables");
  for (int k = 0; k < 2; ++k) alloc((void**)&c->d_jump_tab[k], (size_t)kTpb * kJumpTabWords * 8, "jump tables");
  alloc((void**)&c->d_ranf_window, 110 * 4, "tables");
  alloc((void**)&c->d_err, sizeof(unsigned int), "error word");
  alloc((void**)&c->d_recheck, sizeof(unsigned long long), "recheck counter");
  alloc((void**)&c->d_hist, kMaxBins * kBinStride * sizeof(double), "histogram");
  alloc((void**)&c->d_binw, kMaxBins * sizeof(double), "bin weights");
  alloc((void**)&c->d_adj, kChunk * 10 * sizeof(double), "adjoint sums");
  alloc((void**)&c->d_xo_fe_chunk, 256 * 8, "tables");
  alloc((void**)&c->d_xo_fe_lane, 4 * kFeThreads * 8, "tables");
  alloc((void**)&c->d_fe_lane_tab, (size_t)kFeThreads * kJumpTabWords * 8, "jump tables");
  if (!st) st = c->cuda(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device), "device query");
  alloc(&c->d_state, kChunk * 56 * 4, "batch states");
  (void)dummy;
  (void)p;
  if (!st) st = c->cuda(cudaMemcpy(c->d_xo_batch, t.xo_batch.data(), 256 * 8, cudaMemcpyHostToDevice), "tables");
  if (!st) st = c->cuda(cudaMemcpy(c->d_xo_jump, t.xo_jump.data(), 256 * 8, cudaMemcpyHostToDevice), "tables");
  if (!st) st = c->cuda(cudaMemcpy(c->d_xo_draw, t.xo_draw.data(), 256 * 8, cudaMemcpyHostToDevice), "tables");
  if (!st)
    st = c->cuda(cudaMemcpy(c->d_ranf_tab, t.ranf.data(), kRanfTableRows * 55 * 4, cudaMemcpyHostToDevice), "tables");
  if (!st)
    st = c->cuda(cudaMemcpy(c->d_xo_fe_chunk, t.xo_fe_chunk.data(), 256 * 8, cudaMemcpyHostToDevice), "tables");
  if (!st)
    st = c->cuda(cudaMemcpy(c->d_xo_fe_lane, t.xo_fe_lane.data(), 4 * kFeThreads * 8, cudaMemcpyHostToDevice),
                 "tables");
  if (!st && launch_build_jump_tab(c->d_xo_fe_lane, kFeThreads, c->d_fe_lane_tab, c->stream) != TP_OK)
    st = c->fail(TP_ERR_CUDA, "faster-evgen lane tables: launch failed");
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "faster-evgen lane tables");
  if (!st) st = c->cuda(cudaMemset(c->d_err, 0, sizeof(unsigned int)), "error word");
  if (!st) st = c->cuda(cudaMemset(c->d_recheck, 0, sizeof(unsigned long long)), "recheck counter");
  if (st) {
    g_create_error = c->err;
    if (status) *status = st;
    tp_destroy(c);
    return nullptr;
  }
  if (status) *status = TP_OK;
  return c;
}

void tp_destroy(tp_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  void* bufs[] = {c->d_xo_batch, c->d_xo_jump, c->d_xo_draw, c->d_ranf_tab, c->d_ranf_blocks,
                  c->d_thread_poly[0], c->d_thread_poly[1], c->d_thread_poly[2],
                  c->d_jump_tab[0], c->d_jump_tab[1], c->d_jump_tab[2],
                  c->d_ranf_window, c->d_state, c->d_out, c->d_dump, c->d_err, c->d_recheck,
                  c->d_hist, c->d_binw, c->d_adj, c->d_xo_fe_chunk, c->d_xo_fe_lane, c->d_fe_lane_tab, c->d_fe_chunks,
                  c->d_fe_cstate, c->d_fe_map, c->d_fe_tstate, c->d_fe_store};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (c->h_fe_maps) cudaFreeHost(c->h_fe_maps);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  if (c->pts.exec) cudaGraphExecDestroy(c->pts.exec);
  if (c->pts.graph) cudaGraphDestroy(c->pts.graph);
  if (c->pts.buf) cudaFree(c->pts.buf);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* tp_last_error(const tp_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

int tp_run_batches_async(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch,
                         uint64_t n_batches, int precision, tp_batch_soa* out, void* stream) {
  if (!c) return TP_ERR_INVALID;
  if (!out || !out->selected || !out->spm2 || !out->vars || !out->sigma || !out->variance)
    return c->fail(TP_ERR_INVALID, "null output array");
  cudaSetDevice(c->device);
  BatchOut o{out->selected, out->spm2, out->vars, out->sigma, out->variance, n_batches};
  return run_async(c, cfg, rng_kind, seed, first_batch, n_batches, precision, o,
                   stream ? (cudaStream_t)stream : c->stream);
}

int tp_run_batches(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch,
                   uint64_t n_batches, int precision, tp_batch_soa* out) {
  if (!c) return TP_ERR_INVALID;
  if (!out || !out->selected || !out->spm2 || !out->vars || !out->sigma || !out->variance)
    return c->fail(TP_ERR_INVALID, "null output array");
  if (n_batches == 0) return TP_OK;
  if (n_batches > (1ull << 40)) return c->fail(TP_ERR_INVALID, "batch range too large");
  cudaSetDevice(c->device);
  const size_t n = n_batches;
  if (int st = ensure(c, &c->d_out, &c->out_bytes, n * 13 * 8, "output buffers")) return st;
  auto* sel = static_cast<uint64_t*>(c->d_out);
  auto* f = reinterpret_cast<double*>(sel + n);
  BatchOut o{sel, f, f + 5 * n, f + 10 * n, f + 11 * n, n};
  int st = c->cuda(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), c->stream), "clear error word");
  if (st) return st;
  st = run_async(c, cfg, rng_kind, seed, first_batch, n_batches, precision, o, c->stream);
  if (st) return st;
  st = c->cuda(cudaMemcpyAsync(out->selected, sel, n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  if (!st) st = c->cuda(cudaMemcpyAsync(out->spm2, o.spm2, 5 * n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  if (!st) st = c->cuda(cudaMemcpyAsync(out->vars, o.vars, 5 * n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  if (!st) st = c->cuda(cudaMemcpyAsync(out->sigma, o.sigma, n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  if (!st) st = c->cuda(cudaMemcpyAsync(out->variance, o.variance, n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  unsigned int herr = 0;
  if (!st) st = c->cuda(cudaMemcpyAsync(&herr, c->d_err, sizeof herr, cudaMemcpyDeviceToHost, c->stream), "copy error word");
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "run batches");
  if (!st && herr) return c->fail(TP_ERR_DEVICE, "device error flag " + std::to_string(herr));
  return st;
}

int tp_dump_events(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_event, uint64_t n,
                   tp_event_dump* out) {
  return tp_dump_events_prec(c, cfg, rng_kind, seed, first_event, n, TP_PREC_FP64, out);
}

int tp_dump_events_prec(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_event,
                        uint64_t n, int precision, tp_event_dump* out) {
  if (!c) return TP_ERR_INVALID;
  if (!out) return c->fail(TP_ERR_INVALID, "null output array");
  if (check_config(cfg)) return c->fail(TP_ERR_INVALID, "invalid configuration");
  if (int st = check_kind(c, rng_kind)) return st;
  if (int st = check_seed(c, rng_kind, seed)) return st;
  if (n == 0) return TP_OK;
  if (precision != TP_PREC_FP64 && precision != TP_PREC_FP32_MIXED) return c->fail(TP_ERR_INVALID, "unknown precision");
  if (n > (1ull << 26) || first_event > (1ull << 50)) return c->fail(TP_ERR_INVALID, "dump range too large");
  cudaSetDevice(c->device);
  const bool jpb = (rng_kind & TP_MODE_JUMP_PER_BATCH) != 0;
  if ((rng_kind & TP_RNG_KIND_MASK) == TP_RNG_RANF && !jpb)
    if (int st = ensure_ranf_window(c, (int32_t)seed)) return st;
  if (int st = ensure(c, &c->d_dump, &c->dump_bytes, n * sizeof(tp_event_dump), "dump buffer")) return st;
  EvConst k;
  make_ev_const(*cfg, rng_kind & ~TP_RNG_KIND_MASK, &k);
  uint64_t start[4];
  xoshiro_seed(seed, start);
  int st = c->cuda(cudaMemsetAsync(c->d_err, 0, sizeof(unsigned int), c->stream), "clear error word");
  if (st) return st;
  st = launch_dump(rng_kind, precision, k, start, c->d_ranf_window, (int32_t)seed, c->d_xo_draw, c->d_xo_jump, c->d_ranf_tab,
                   first_event, n, static_cast<tp_event_dump*>(c->d_dump), c->d_err, c->stream);
  if (st) return c->fail(st, std::string("dump launch: ") + cudaGetErrorString(cudaGetLastError()));
  unsigned int herr = 0;
  st = c->cuda(cudaMemcpyAsync(out, c->d_dump, n * sizeof(tp_event_dump), cudaMemcpyDeviceToHost, c->stream), "copy dump");
  if (!st) st = c->cuda(cudaMemcpyAsync(&herr, c->d_err, sizeof herr, cudaMemcpyDeviceToHost, c->stream), "copy error word");
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "dump events");
  if (!st && herr) return c->fail(TP_ERR_UNSUPPORTED, "ranf batch seed outside [0, 1e9): no jump-ahead");
  return st;
}

int tp_set_fe_store_cap(tp_ctx* c, uint64_t bytes) {
  if (!c) return TP_ERR_INVALID;
  c->fe_store_cap = bytes;
  return TP_OK;
}

int tp_set_events_per_thread(tp_ctx* c, int ept) {
  if (!c) return TP_ERR_INVALID;
  if (ept <= 0 || (TP_BATCH_SIZE + ept - 1) / ept > kTpb) return c->fail(TP_ERR_INVALID, "events per thread out of range");
  c->ept[0] = c->ept[1] = c->ept[2] = ept;
  return TP_OK;
}

int tp_binned_forward(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch,
                      uint64_t n_batches, int precision, const tp_binning* bins, double* out) {
  if (!c) return TP_ERR_INVALID;
  if (!out) return c->fail(TP_ERR_INVALID, "null output array");
  if (check_config(cfg)) return c->fail(TP_ERR_INVALID, "invalid configuration");
  cudaSetDevice(c->device);
  KParams kp{};
  if (int st = binning_params(c, cfg, bins, &kp)) return st;
  const size_t nbin = (size_t)kp.nx * kp.ny;
  int st = c->cuda(cudaMemsetAsync(c->d_hist, 0, nbin * kBinStride * sizeof(double), c->stream), "clear histogram");
  if (st) return st;
  BatchOut none{};
  st = run_async(c, cfg, rng_kind, seed, first_batch, n_batches, precision, none, c->stream, Pass::kBinned, &kp);
  if (st) return st;
  st = c->cuda(cudaMemcpyAsync(out, c->d_hist, nbin * kBinStride * sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream), "copy histogram");
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "binned forward");
  return st;
}

int tp_binned_adjoint(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch,
                      uint64_t n_batches, int precision, const tp_binning* bins, const double* bin_weight,
                      double g[5], double s_out[5]) {
  if (!c) return TP_ERR_INVALID;
  if (!bin_weight || !g || !s_out) return c->fail(TP_ERR_INVALID, "null array");
  if (check_config(cfg)) return c->fail(TP_ERR_INVALID, "invalid configuration");
  cudaSetDevice(c->device);
  KParams kp{};
  if (int st = binning_params(c, cfg, bins, &kp)) return st;
  const size_t nbin = (size_t)kp.nx * kp.ny;
  int st = c->cuda(cudaMemcpyAsync(c->d_binw, bin_weight, nbin * sizeof(double), cudaMemcpyHostToDevice, c->stream),
                   "upload bin weights");
  if (st) return st;
  std::vector<double> per_batch;
  per_batch.reserve(10 * (n_batches < kChunk ? n_batches : kChunk));
  BatchOut none{};
  st = run_async(c, cfg, rng_kind, seed, first_batch, n_batches, precision, none, c->stream, Pass::kAdjoint, &kp,
                 &per_batch);
  if (st) return st;
  for (int k = 0; k < 5; ++k) g[k] = s_out[k] = 0.0;
  for (uint64_t i = 0; i < n_batches; ++i)  // batch order
    for (int k = 0; k < 5; ++k) {
      g[k] += per_batch[10 * i + k];
      s_out[k] += per_batch[10 * i + 5 + k];
    }
  return TP_OK;
}

int tp_grad(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch, uint64_t n_batches,
            int precision, const tp_binning* bins, const double* bin_weight, double dlnl_dtheta[4],
            double dsigma_dtheta[4]) {
  if (!c) return TP_ERR_INVALID;
  double g[5], sg[5], k[5], dk[20], flux = 0.0;
  if (int st = tp_binned_adjoint(c, cfg, rng_kind, seed, first_batch, n_batches, precision, bins, bin_weight, g, sg))
    return st;
  if (int st = tp_coupling_factors(cfg, k, dk, &flux)) return c->fail(st, "coupling factors");
  for (int i = 0; i < 4; ++i) {
    double a = 0.0, b = 0.0;
    for (int q = 0; q < 5; ++q) {
      a += g[q] * dk[4 * q + i];
      b += sg[q] * dk[4 * q + i];
    }
    if (dlnl_dtheta) dlnl_dtheta[i] = flux * a;
    if (dsigma_dtheta) dsigma_dtheta[i] = flux * b;
  }
  return TP_OK;
}

namespace {

// tp_run_points and tp_run_points_ranf: `starts` holds xoshiro states
// (4 x u64 per point) or ranf seeds (one i32 per point).
int run_points(tp_ctx* c, int kind, uint32_t n_points, const tp_config* cfgs, const void* starts, int mode_flags,
               int precision, uint64_t* unit0, tp_batch_soa* out, uint64_t capacity) {
  if (!c) return TP_ERR_INVALID;
  if (!cfgs || !starts || !unit0 || !out || !out->selected || !out->spm2 || !out->vars || !out->sigma ||
      !out->variance)
    return c->fail(TP_ERR_INVALID, "null array");
  if (n_points == 0 || n_points > (1u << 20)) return c->fail(TP_ERR_INVALID, "n_points out of range");
  if (mode_flags & ~TP_MODE_NO_PHOTON_SORTING) return c->fail(TP_ERR_INVALID, "unsupported mode flag");
  if (precision != TP_PREC_FP64 && precision != TP_PREC_FP32_MIXED) return c->fail(TP_ERR_INVALID, "unknown precision");
  cudaSetDevice(c->device);
  // units: every point's batches, point by point
  std::vector<EvConst> pk(n_points);
  std::vector<uint64_t> pev(n_points);
  uint64_t n_units = 0;
  for (uint32_t p = 0; p < n_points; ++p) {
    if (check_config(&cfgs[p])) return c->fail(TP_ERR_INVALID, "invalid configuration of point " + std::to_string(p));
    make_ev_const(cfgs[p], mode_flags, &pk[p]);
    pev[p] = cfgs[p].num_events;
    unit0[p] = n_units;
    n_units += (cfgs[p].num_events + kBatch - 1) / kBatch;
  }
  unit0[n_points] = n_units;
  if (n_units > capacity) return c->fail(TP_ERR_INVALID, "output capacity below the number of batches");
  if (n_units > (1ull << 31)) return c->fail(TP_ERR_INVALID, "too many batches");
  std::vector<uint32_t> unit_point(n_units);
  for (uint32_t p = 0; p < n_points; ++p)
    for (uint64_t u = unit0[p]; u < unit0[p + 1]; ++u) unit_point[u] = p;
  const int pi = prec_index(precision);
  const bool ranf = kind == TP_RNG_RANF;
  // ranf: each point's stream from its seed (blocks 0 and 1, the window
  // every batch start is jumped from)
  std::vector<int32_t> windows;
  if (ranf) {
    if (int st = ensure_ranf_blocks(c)) return st;
    windows.resize(110 * (size_t)n_points);
    const int32_t* seeds = static_cast<const int32_t*>(starts);
    for (uint32_t p = 0; p < n_points; ++p) {
      int32_t* w = windows.data() + 110 * (size_t)p;
      ranf_seeded(seeds[p], w);
      if (!ranf_canonical(w))
        return c->fail(TP_ERR_UNSUPPORTED, "ranf seed of point " + std::to_string(p) +
                                               " gives a state outside [0, 1e9): no jump-ahead");
      for (int i = 0; i < 55; ++i) w[55 + i] = w[i];
      ranf_reset(w + 55);
    }
  } else if (int st = ensure_thread_poly(c, pi)) {
    return st;
  }
  // one device buffer, 256-byte aligned sections
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t start_bytes = ranf ? n_points * 110 * sizeof(int32_t) : n_points * 32;
  const size_t state_bytes = ranf ? 56 * sizeof(int32_t) : 32;
  const size_t o_pts = 0, o_ev = o_pts + al(n_points * sizeof(EvConst)), o_u0 = o_ev + al(n_points * 8),
               o_st = o_u0 + al(n_points * 8), o_up = o_st + al(start_bytes), o_us = o_up + al(n_units * 4),
               o_out = o_us + al(n_units * state_bytes), o_cnt = o_out + al(n_units * 13 * 8), total = o_cnt + 256;
  if (c->pts.bytes < total) {
    if (c->pts.buf) cudaFree(c->pts.buf);
    c->pts.buf = nullptr;
    c->pts.bytes = 0;
    if (int st = c->cuda(cudaMalloc(&c->pts.buf, total), "points buffers")) return st;
    c->pts.bytes = total;
  }
  char* base = static_cast<char*>(c->pts.buf);
  PointsParams pp{};
  pp.kind = kind;
  pp.points = reinterpret_cast<const EvConst*>(base + o_pts);
  pp.point_events = reinterpret_cast<const uint64_t*>(base + o_ev);
  pp.point_unit0 = reinterpret_cast<const uint64_t*>(base + o_u0);
  pp.point_start = reinterpret_cast<const uint64_t*>(base + o_st);
  pp.point_window = reinterpret_cast<const int32_t*>(base + o_st);
  pp.unit_point = reinterpret_cast<const uint32_t*>(base + o_up);
  pp.unit_state = base + o_us;
  pp.batch_table = c->d_xo_batch;
  pp.ranf_table = c->d_ranf_tab;
  pp.ranf_blocks = c->d_ranf_blocks;
  pp.thread_poly = c->d_thread_poly[pi];
  pp.jump_tab = c->d_jump_tab[pi];
  pp.counter = reinterpret_cast<unsigned long long*>(base + o_cnt);
  pp.recheck_count = c->d_recheck;
  auto* sel = reinterpret_cast<uint64_t*>(base + o_out);
  auto* f = reinterpret_cast<double*>(sel + n_units);
  pp.out = BatchOut{sel, f, f + 5 * n_units, f + 10 * n_units, f + 11 * n_units, n_units};
  pp.n_units = n_units;
  pp.ept = c->ept[pi];
  pp.precision = precision;
  pp.occupancy = c->occupancy[pi];
  int st = TP_OK;
  auto up = [&](size_t off, const void* src, size_t n) {
    if (!st) st = c->cuda(cudaMemcpyAsync(base + off, src, n, cudaMemcpyHostToDevice, c->stream), "upload points");
  };
  up(o_pts, pk.data(), n_points * sizeof(EvConst));
  up(o_ev, pev.data(), n_points * 8);
  up(o_u0, unit0, n_points * 8);
  up(o_st, ranf ? (const void*)windows.data() : starts, start_bytes);
  up(o_up, unit_point.data(), n_units * 4);
  if (st) return st;
  // the seeding + persistent launches are captured once per shape and replayed
  const uint64_t key[8] = {n_points, n_units, (uint64_t)precision, (uint64_t)pp.ept, (uint64_t)mode_flags,
                           (uint64_t)(uintptr_t)c->pts.buf, (uint64_t)pp.occupancy, (uint64_t)kind};
  if (!c->pts.exec || std::memcmp(key, c->pts.key, sizeof key) != 0) {
    if (c->pts.exec) cudaGraphExecDestroy(c->pts.exec);
    if (c->pts.graph) cudaGraphDestroy(c->pts.graph);
    c->pts.exec = nullptr;
    c->pts.graph = nullptr;
    const int need = (kBatch + pp.ept - 1) / pp.ept;
    const int tpb = ((need + 31) / 32) * 32;
    st = c->cuda(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
    if (st) return st;
    cudaMemsetAsync(pp.counter, 0, sizeof(unsigned long long), c->stream);
    const int lst = launch_points(pp, tpb, c->stream);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
    if (lst || ce != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return c->fail(TP_ERR_CUDA, "capturing the points launch failed");
    }
    st = c->cuda(cudaGraphInstantiate(&c->pts.exec, g, 0), "graph instantiate");
    if (st) {
      cudaGraphDestroy(g);
      return st;
    }
    c->pts.graph = g;
    std::memcpy(c->pts.key, key, sizeof key);
  }
  if (c->prof) {
    cudaEvent_t e0 = c->next_event(), e1 = c->next_event();
    if (e0 && e1) {
      cudaEventRecord(e0, c->stream);
      st = c->cuda(cudaGraphLaunch(c->pts.exec, c->stream), "graph launch");
      cudaEventRecord(e1, c->stream);
      c->prof_marks.push_back({1, {e0, e1}});
    }
  } else {
    st = c->cuda(cudaGraphLaunch(c->pts.exec, c->stream), "graph launch");
  }
  if (st) return st;
  const size_t n = n_units;
  st = c->cuda(cudaMemcpyAsync(out->selected, sel, n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  if (!st) st = c->cuda(cudaMemcpyAsync(out->spm2, pp.out.spm2, 5 * n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  if (!st) st = c->cuda(cudaMemcpyAsync(out->vars, pp.out.vars, 5 * n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  if (!st) st = c->cuda(cudaMemcpyAsync(out->sigma, pp.out.sigma, n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  if (!st) st = c->cuda(cudaMemcpyAsync(out->variance, pp.out.variance, n * 8, cudaMemcpyDeviceToHost, c->stream), "copy results");
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "run points");
  return st;
}

}  // namespace

int tp_run_points(tp_ctx* c, uint32_t n_points, const tp_config* cfgs, const uint64_t* starts, int mode_flags,
                  int precision, uint64_t* unit0, tp_batch_soa* out, uint64_t capacity) {
  return run_points(c, TP_RNG_XOSHIRO256P, n_points, cfgs, starts, mode_flags, precision, unit0, out, capacity);
}

int tp_run_points_ranf(tp_ctx* c, uint32_t n_points, const tp_config* cfgs, const int32_t* seeds, int mode_flags,
                       int precision, uint64_t* unit0, tp_batch_soa* out, uint64_t capacity) {
  return run_points(c, TP_RNG_RANF, n_points, cfgs, seeds, mode_flags, precision, unit0, out, capacity);
}

int tp_autotune(tp_ctx* c, const tp_config* cfg, int precision, uint64_t sample_batches, int* best_ept,
                double* best_events_per_s) {
  if (!c) return TP_ERR_INVALID;
  if (check_config(cfg)) return c->fail(TP_ERR_INVALID, "invalid configuration");
  if (sample_batches == 0 || sample_batches > kChunk) return c->fail(TP_ERR_INVALID, "sample_batches out of range");
  cudaSetDevice(c->device);
  // events per thread -> threads per CTA = ceil(10000 / ept) rounded to
  // warps (more events per thread: fewer per-thread stream jumps of 256
  // steps). The candidates fill their last warp: ceil(10000 / ept) is at
  // or just below 256, 192, 160, 128, 96, 64 and 32 threads.
  static const int candidates[] = {40, 53, 63, 79, 105, 157, 313};
  const size_t n = sample_batches;
  if (int st = ensure(c, &c->d_out, &c->out_bytes, n * 13 * 8, "output buffers")) return st;
  auto* sel = static_cast<uint64_t*>(c->d_out);
  auto* f = reinterpret_cast<double*>(sel + n);
  BatchOut o{sel, f, f + 5 * n, f + 10 * n, f + 11 * n, n};
  cudaEvent_t a = c->next_event(), b = c->next_event();
  const int pi = precision == TP_PREC_FP32_MIXED ? 1 : 0;
  const int saved = c->ept[pi], saved_occ = c->occupancy[pi];
  double best_t = 1e300;
  int best = saved, best_occ = saved_occ;
  // occupancy variants: FP64 2 or 3 CTAs per SM, FP32-mixed 2, 3 or 4
  const int n_occ = precision == TP_PREC_FP32_MIXED ? 3 : 2;
  for (int cand = 0; cand < n_occ * (int)(sizeof candidates / sizeof candidates[0]); ++cand) {
    const int ept = candidates[cand / n_occ];
    const int occ = 2 + cand % n_occ;
    c->ept[pi] = ept;
    c->occupancy[pi] = occ;
    // whole waves of resident CTAs, so that a candidate whose last wave
    // the sample happens to leave nearly empty is not penalised for it
    const int tpb = (((int)kBatch + ept - 1) / ept + 31) / 32 * 32;
    const uint64_t wave = (uint64_t)events_wave(precision, occ, tpb);
    const uint64_t ns = n >= wave ? n / wave * wave : n;
    int st = run_async(c, cfg, TP_RNG_XOSHIRO256P, 12345, 0, ns, precision, o, c->stream);  // warm-up
    if (st) {
      c->ept[pi] = saved;
      c->occupancy[pi] = saved_occ;
      return st;
    }
    // the fastest of three separately timed runs (a sample takes about a
    // millisecond, so single timings are noisy)
    float ms = 1e30f;
    for (int rep = 0; rep < 3 && !st; ++rep) {
      cudaEventRecord(a, c->stream);
      st = run_async(c, cfg, TP_RNG_XOSHIRO256P, 12345, 0, ns, precision, o, c->stream);
      cudaEventRecord(b, c->stream);
      if (!st) st = c->cuda(cudaEventSynchronize(b), "autotune");
      float one = 0.f;
      if (!st) cudaEventElapsedTime(&one, a, b);
      if (one < ms) ms = one;
    }
    if (st) {
      c->ept[pi] = saved;
      c->occupancy[pi] = saved_occ;
      return st;
    }
    const double t = ms / (double)ns;  // per batch
    if (t < best_t) {
      best_t = t;
      best = ept;
      best_occ = occ;
    }
  }
  c->ev_used = 0;
  c->ept[pi] = best;
  c->occupancy[pi] = best_occ;
  if (best_ept) *best_ept = best;
  if (best_events_per_s) *best_events_per_s = (double)kBatch / (best_t * 1e-3);
  return TP_OK;
}

int tp_get_tuning(tp_ctx* c, int precision, int* ept, int* min_ctas_per_sm) {
  if (!c) return TP_ERR_INVALID;
  if (precision != TP_PREC_FP64 && precision != TP_PREC_FP32_MIXED)
    return c->fail(TP_ERR_INVALID, "unknown precision");
  if (ept) *ept = c->ept[prec_index(precision)];
  if (min_ctas_per_sm) *min_ctas_per_sm = c->occupancy[precision == TP_PREC_FP32_MIXED ? 1 : 0];
  return TP_OK;
}

int tp_set_occupancy(tp_ctx* c, int precision, int min_ctas_per_sm) {
  if (!c) return TP_ERR_INVALID;
  if (precision != TP_PREC_FP64 && precision != TP_PREC_FP32_MIXED)
    return c->fail(TP_ERR_INVALID, "unknown precision");
  const int hi = precision == TP_PREC_FP32_MIXED ? 4 : 3;
  if (min_ctas_per_sm < 2 || min_ctas_per_sm > hi)
    return c->fail(TP_ERR_INVALID, "min_ctas_per_sm: 2 or 3 (FP64), 2 to 4 (FP32-mixed)");
  c->occupancy[precision == TP_PREC_FP32_MIXED ? 1 : 0] = min_ctas_per_sm;
  return TP_OK;
}

int tp_fp32_error(tp_ctx* c, const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch,
                  uint64_t n_batches, double* err_vs_fp64, tp_batch_soa* fp32, tp_batch_soa* fp64) {
  if (!c) return TP_ERR_INVALID;
  if (!err_vs_fp64) return c->fail(TP_ERR_INVALID, "null output array");
  if (n_batches == 0) return TP_OK;
  if (n_batches > (1ull << 32)) return c->fail(TP_ERR_INVALID, "batch range too large");
  const size_t n = n_batches;
  std::vector<uint64_t> sel[2] = {std::vector<uint64_t>(n), std::vector<uint64_t>(n)};
  std::vector<double> f[2] = {std::vector<double>(12 * n), std::vector<double>(12 * n)};
  tp_batch_soa soa[2];
  for (int k = 0; k < 2; ++k) {
    soa[k] = tp_batch_soa{sel[k].data(), f[k].data(), f[k].data() + 5 * n, f[k].data() + 10 * n,
                          f[k].data() + 11 * n};
    const int precision = k == 0 ? TP_PREC_FP32_MIXED : TP_PREC_FP64;
    if (int st = tp_run_batches(c, cfg, rng_kind, seed, first_batch, n_batches, precision, &soa[k])) return st;
  }
  for (size_t i = 0; i < n; ++i) {
    if (sel[0][i] != sel[1][i]) {
      err_vs_fp64[i] = -1.0;
      continue;
    }
    double e = 0.0;
    const double scale_a = std::fabs(f[1][i]);  // spm2[0]: the A sum
    for (int q = 0; q < 12; ++q) {
      const double a = f[0][q * n + i], b = f[1][q * n + i];
      // the mixed terms (spm2[3], spm2[4]) cancel: their natural scale is A's
      const double scale = (q == 3 || q == 4) ? std::fmax(std::fabs(b), scale_a) : std::fabs(b);
      if (scale > 0.0) e = std::fmax(e, std::fabs(a - b) / scale);
      else if (a != 0.0) e = std::fmax(e, 1.0);
    }
    err_vs_fp64[i] = e;
  }
  tp_batch_soa* outs[2] = {fp32, fp64};
  for (int k = 0; k < 2; ++k) {
    tp_batch_soa* o = outs[k];
    if (!o) continue;
    if (o->selected) std::memcpy(o->selected, sel[k].data(), n * 8);
    if (o->spm2) std::memcpy(o->spm2, soa[k].spm2, 5 * n * 8);
    if (o->vars) std::memcpy(o->vars, soa[k].vars, 5 * n * 8);
    if (o->sigma) std::memcpy(o->sigma, soa[k].sigma, n * 8);
    if (o->variance) std::memcpy(o->variance, soa[k].variance, n * 8);
  }
  return TP_OK;
}

int tp_recheck_count(tp_ctx* c, uint64_t* count, int reset) {
  if (!c || !count) return TP_ERR_INVALID;
  cudaSetDevice(c->device);
  unsigned long long h = 0;
  int st = c->cuda(cudaMemcpyAsync(&h, c->d_recheck, sizeof h, cudaMemcpyDeviceToHost, c->stream), "recheck counter");
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "recheck counter");
  if (!st && reset) st = c->cuda(cudaMemset(c->d_recheck, 0, sizeof h), "recheck counter");
  if (!st) *count = h;
  return st;
}

int tp_profile(tp_ctx* c, int enable) {
  if (!c) return TP_ERR_INVALID;
  cudaSetDevice(c->device);
  if (enable) {
    c->prof_marks.clear();
    c->ev_used = 0;
  }
  c->prof = enable ? 1 : 0;
  return TP_OK;
}

int tp_profile_read(tp_ctx* c, double* event_ms, uint64_t* event_launches, double* seed_ms, uint64_t* seed_launches) {
  if (!c) return TP_ERR_INVALID;
  cudaSetDevice(c->device);
  double ms[2] = {0.0, 0.0};
  uint64_t cnt[2] = {0, 0};
  for (auto& m : c->prof_marks) {
    if (int st = c->cuda(cudaEventSynchronize(m.second.second), "profile")) return st;
    float t = 0.f;
    if (int st = c->cuda(cudaEventElapsedTime(&t, m.second.first, m.second.second), "profile")) return st;
    ms[m.first] += t;
    cnt[m.first] += 1;
  }
  if (event_ms) *event_ms = ms[1];
  if (event_launches) *event_launches = cnt[1];
  if (seed_ms) *seed_ms = ms[0];
  if (seed_launches) *seed_launches = cnt[0];
  c->prof_marks.clear();
  c->ev_used = 0;
  return TP_OK;
}

namespace {
// seconds per operation of k_probe's op `op` (chains per thread: 16 for the
// FMA ops 0 and 5, else 8), timed until a launch lasts 20 ms. One untimed
// launch comes first: the first launch of a kernel also loads its module
// (lazy loading), which can take longer than the 20 ms mark by itself.
int probe_op_seconds(tp_ctx* c, int op, double* seconds) {
  int sms = 0;
  if (int st = c->cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device), "probe")) return st;
  double* sink = nullptr;
  if (int st = c->cuda(cudaMalloc(&sink, sizeof(double)), "probe")) return st;
  cudaEvent_t a = c->next_event(), b = c->next_event();
  const int blocks = sms * 8, tpb = 256;
  const double threads = (double)blocks * tpb;
  const double chains = (op == 0 || op == 5) ? 16.0 : 8.0;
  int st = launch_probe(op, 1, blocks, tpb, sink, c->stream);
  if (!st) st = c->cuda(cudaStreamSynchronize(c->stream), "probe");
  int iters = 16;
  for (int rep = 0; rep < 8 && !st; ++rep) {
    cudaEventRecord(a, c->stream);
    st = launch_probe(op, iters, blocks, tpb, sink, c->stream);
    cudaEventRecord(b, c->stream);
    if (!st) st = c->cuda(cudaEventSynchronize(b), "probe");
    if (st) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (ms > 20.f || rep == 7) {
      *seconds = (ms * 1e-3) / (threads * chains * iters);
      break;
    }
    const double grow = ms > 0.01f ? 25.0 / ms : 64.0;
    iters = (int)(iters * (grow > 64.0 ? 64.0 : grow)) + 1;
  }
  cudaFree(sink);
  c->ev_used = 0;
  return st;
}
}  // namespace

int tp_probe_fp32(tp_ctx* c, double out[2]) {
  if (!c || !out) return TP_ERR_INVALID;
  cudaSetDevice(c->device);
  double ffma = 0.0, mufu = 0.0;
  if (int st = probe_op_seconds(c, 5, &ffma)) return st;
  if (int st = probe_op_seconds(c, 6, &mufu)) return st;
  out[0] = 2.0 / ffma;  // FP32 flop/s, an FMA counting 2
  out[1] = 1.0 / mufu;  // special-function operations/s (log2, each with one add)
  return TP_OK;
}

int tp_probe_fp64(tp_ctx* c, double out[5]) {
  if (!c || !out) return TP_ERR_INVALID;
  cudaSetDevice(c->device);
  double per_op_s[5];
  for (int op = 0; op < 5; ++op)
    if (int st = probe_op_seconds(c, op, &per_op_s[op])) return st;
  out[0] = 2.0 / per_op_s[0];  // DFMA flop/s
  for (int op = 1; op < 5; ++op) out[op] = per_op_s[op] / per_op_s[0];  // DFMA equivalents
  return TP_OK;
}

// ---- host-side jump-ahead (no GPU) ----
int tp_xoshiro_state_at(uint64_t seed, uint64_t jumps128, uint64_t draws, uint64_t state[4]) {
  if (!state) return TP_ERR_INVALID;
  xoshiro_seed(seed, state);
  if (jumps128) {
    const Tables& t = host_tables();
    for (int k = 0; k < 64; ++k)
      if ((jumps128 >> k) & 1) {
        Gf2Poly p;
        for (int w = 0; w < 4; ++w) p.w[w] = t.xo_jump[4 * k + w];
        xoshiro_apply(p, state);
      }
  }
  if (draws) xoshiro_apply(gf2_xpow(draws), state);
  return TP_OK;
}

int tp_ranf_state_at(int32_t seed, uint64_t draws, int32_t slots[55], int32_t* index) {
  if (!slots || !index) return TP_ERR_INVALID;
  int32_t w[110];
  ranf_seeded(seed, w);
  if (!ranf_canonical(w)) return TP_ERR_UNSUPPORTED;
  for (int i = 0; i < 55; ++i) w[55 + i] = w[i];
  ranf_reset(w + 55);
  const uint64_t r = draws / 55, m = draws % 55;
  ranf_apply(ranf_xpow(55 * r), w, slots);
  *index = (int32_t)(55 - m);
  return TP_OK;
}

}  // extern "C"
