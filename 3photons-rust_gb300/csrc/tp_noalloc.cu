// tp_noalloc.cu — tp_run_batches_noalloc: the batch event loop for callers
// that must not allocate GPU memory.
//
// Some hosts cannot call cudaMalloc at the moment they want events:
// real-time or embedded callers whose GPU memory is planned once at
// start-up, or programs whose GPU memory belongs to another allocator (a
// framework's caching pool) that the library must not bypass. This entry
// point serves them: it needs no tp_ctx, calls no cudaMalloc/cudaFree, and
// keeps its only working memory in the fixed arrays below, which exist on
// every GPU that loads the library for as long as the process lives.
//
// Working memory: the start state of every batch of the call (the scratch
// written by the seeding kernel and read by the event kernel), plus the
// jump-ahead polynomials both kernels read. The event kernels are the same
// ones tp_run_batches_async launches.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "tp_internal.h"
#include "tp_rng.h"

namespace tp {
namespace {

constexpr int kNoallocEpt = 40;   // events per thread of these launches
constexpr int kNoallocTpb = 256;  // ceil(10000 / 40) = 250 threads, in warps

// Batch start states: 4 x u64 per batch.
static __device__ __align__(256) uint64_t g_noalloc_state[4 * TP_NOALLOC_MAX_BATCHES];
// Jump polynomials (4 words each): [0, 64) x^(12e4 * 2^k) for one-stream
// runs, [64, 128) x^(2^(128 + k)) for the per-batch jump, [128, 384)
// x^(12 * 40 * j) for thread j of a batch.
static __device__ __align__(256) uint64_t g_noalloc_tables[4 * 384];

struct DeviceSetup {
  bool ready = false;
  unsigned long long ctx_id = 0;  // the CUDA context the addresses belong to
  uint64_t* state = nullptr;      // device address of g_noalloc_state
  uint64_t* tables = nullptr;     // device address of g_noalloc_tables
};

constexpr int kMaxDevices = 64;
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mutex;
// messages go where tp_last_error(NULL) reads them
int fail(int code, const char* msg) {
  set_thread_error(msg);
  return code;
}

// The process-unique ID of the current CUDA context (cuCtxGetId through
// the runtime's driver entry points, so the library links no driver
// library), or 0 when it cannot be read. A cudaDeviceReset followed by new
// work gives the device a new primary context with a new ID, whose copy of
// the fixed arrays has not been set up.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

// Once per device and context, with that device current: look up the
// arrays' device addresses and upload the jump polynomials (a plain copy
// into the fixed array; nothing is allocated). The lookup also makes the
// device's primary context current on this thread.
int setup_device(int dev, DeviceSetup** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  DeviceSetup& d = g_setup[dev];
  void* state = nullptr;
  void* tables = nullptr;
  if (cudaGetSymbolAddress(&state, g_noalloc_state) != cudaSuccess ||
      cudaGetSymbolAddress(&tables, g_noalloc_tables) != cudaSuccess)
    return fail(TP_ERR_CUDA, "tp_run_batches_noalloc: cudaGetSymbolAddress failed on this device");
  const unsigned long long ctx_id = current_context_id();
  if (!d.ready || (ctx_id != 0 && ctx_id != d.ctx_id) || state != d.state || tables != d.tables) {
    d.ready = false;
    uint64_t host[4 * 384];
    Gf2Poly pb = gf2_xpow(kDrawsPerBatch), pj = gf2_xpow2k(128);
    for (int k = 0; k < 64; ++k) {
      for (int w = 0; w < 4; ++w) {
        host[4 * k + w] = pb.w[w];
        host[4 * (64 + k) + w] = pj.w[w];
      }
      pb = gf2_mulmod(pb, pb);
      pj = gf2_mulmod(pj, pj);
    }
    const Gf2Poly step = gf2_xpow((uint64_t)kDrawsPerEvent * kNoallocEpt);
    Gf2Poly cur{{1, 0, 0, 0}};
    for (int j = 0; j < 256; ++j) {
      for (int w = 0; w < 4; ++w) host[4 * (128 + j) + w] = cur.w[w];
      cur = gf2_mulmod(cur, step);
    }
    if (cudaMemcpy(tables, host, sizeof host, cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(TP_ERR_CUDA, "tp_run_batches_noalloc: uploading the jump tables failed");
    d.state = static_cast<uint64_t*>(state);
    d.tables = static_cast<uint64_t*>(tables);
    d.ctx_id = ctx_id;
    d.ready = true;
  }
  *out = &d;
  return TP_OK;
}

}  // namespace
}  // namespace tp

using namespace tp;

extern "C" int tp_run_batches_noalloc(const tp_config* cfg, int rng_kind, uint64_t seed, uint64_t first_batch,
                                      uint64_t n_batches, int precision, tp_batch_soa* out, void* stream) {
  if (check_config(cfg)) return fail(TP_ERR_INVALID, "tp_run_batches_noalloc: invalid configuration");
  if ((rng_kind & TP_RNG_KIND_MASK) != TP_RNG_XOSHIRO256P ||
      (rng_kind & ~(TP_RNG_KIND_MASK | TP_MODE_JUMP_PER_BATCH | TP_MODE_NO_PHOTON_SORTING)))
    return fail(TP_ERR_INVALID, "tp_run_batches_noalloc: rng_kind must be TP_RNG_XOSHIRO256P (+ mode flags)");
  if (precision != TP_PREC_FP64 && precision != TP_PREC_FP32_MIXED)
    return fail(TP_ERR_INVALID, "tp_run_batches_noalloc: unknown precision");
  if (!out || !out->selected || !out->spm2 || !out->vars || !out->sigma || !out->variance)
    return fail(TP_ERR_INVALID, "tp_run_batches_noalloc: null output array");
  if (n_batches == 0) return TP_OK;
  if (n_batches > TP_NOALLOC_MAX_BATCHES)
    return fail(TP_ERR_INVALID,
                "tp_run_batches_noalloc: n_batches exceeds TP_NOALLOC_MAX_BATCHES (4096); split the range into "
                "several calls");
  if (first_batch > (1ull << 46)) return fail(TP_ERR_INVALID, "tp_run_batches_noalloc: first_batch too large");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(TP_ERR_NO_DEVICE, "tp_run_batches_noalloc: no current CUDA device");
  DeviceSetup* d = nullptr;
  if (int st = setup_device(dev, &d)) return st;

  KParams kp{};
  make_ev_const(*cfg, rng_kind & ~TP_RNG_KIND_MASK, &kp.k);
  kp.first_batch = first_batch;
  kp.n_batches = n_batches;
  kp.num_events = cfg->num_events;
  kp.ept = kNoallocEpt;
  kp.precision = precision;
  kp.batch_state = d->state;
  kp.thread_poly = d->tables + 4 * 128;
  kp.out = BatchOut{out->selected, out->spm2, out->vars, out->sigma, out->variance, n_batches};
  uint64_t start[4];
  xoshiro_seed(seed, start);
  const bool jpb = (rng_kind & TP_MODE_JUMP_PER_BATCH) != 0;
  if (launch_seed_xoshiro(start, d->tables + (jpb ? 4 * 64 : 0), first_batch, n_batches, d->state, stream) != TP_OK)
    return fail(TP_ERR_CUDA, "tp_run_batches_noalloc: seeding launch failed");
  if (launch_events(rng_kind, kp, kNoallocTpb, stream) != TP_OK)
    return fail(TP_ERR_CUDA, "tp_run_batches_noalloc: event launch failed");
  return TP_OK;
}
