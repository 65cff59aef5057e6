// Host side of the propagation engine: the C ABI of include/cpgpu.h, network
// upload, the device level stack, AC / SAC orchestration, and the MAC and
// GModelSolver search loops that keep the reference's host control flow while
// every domain operation and propagation runs on the device.
#include <sys/stat.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cpgpu.h"
#include "cp_gen.h"
#include "cp_internal.h"

using namespace cpgpu;

// Threads per CTA of the tiled SAC sweep (one tile of 32 branches per CTA).
constexpr int kTileBlock = 256;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define CP_CUDA(expr)                                                                          \
  do {                                                                                         \
    cudaError_t _e = (expr);                                                                   \
    if (_e != cudaSuccess) {                                                                   \
      const int _code = (_e == cudaErrorMemoryAllocation) ? CP_E_OOM : CP_E_CUDA;              \
      return fail(_code, std::string(#expr) + ": " + cudaGetErrorString(_e));                  \
    }                                                                                          \
  } while (0)

#define CP_TRY(expr)          \
  do {                        \
    int _r = (expr);          \
    if (_r != CP_OK) return _r; \
  } while (0)

int internal_words(int W) {
  if (W <= 2) return W;
  if (W <= 4) return 4;
  if (W <= 8) return 8;
  return -1;
}

}  // namespace

void cpgpu::set_last_error(const std::string& msg) { g_last_error = msg; }

struct cp_engine {
  int device = 0;
  cudaStream_t stream = nullptr;
  // Asynchronous reloads: copies and the derivation of the other relation
  // side run on a lowest-priority stream; the engine's stream waits on xfer_ev.
  cudaStream_t xfer = nullptr;
  cudaEvent_t xfer_ev = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evk0 = nullptr, evk1 = nullptr;
  int sm_count = 0;
  size_t smem_optin = 0;
  int64_t launches = 0;
  int live_nets = 0;
  bool closed = false;
  int block_node = 256;
  int block_sac = 256;
  int chunk = 0;
  int ctas_per_sm = 0;
  int sac_mode = 0;  // 0: tiled sweep where eligible, 1: general kernel only
  bool sac_graphs = true;  // single-network SAC1 rounds replayed as CUDA graphs
  int cta_quota = 0;  // batch sweep CTAs retire after this many units (0: persistent)
  int search_mode = 0;  // 0: MAC searches run on the device where they fit one CTA; 1: host-driven nodes
  int search_block = 0;  // threads per search CTA, 0: chosen per launch
  long long wait_ns = 2000000000ll;  // longest grid-barrier wait of a block (then CP_E_TIMEOUT)
  int64_t fail_alloc_after = -1;     // test hook: device allocations left before one fails (-1: off)
  std::multimap<size_t, void*> mapped_free;  // host-mapped pinned blocks (device-written results)
  int priority = 0;   // stream priority class: -1 low, 0 default, 1 high
  // Device memory of this engine's networks and batches comes from a
  // stream-ordered pool on the engine stream: allocation is a sub-allocation
  // and release does not synchronise the device, which keeps per-request
  // upload and teardown cheap while other streams run.
  cudaMemPool_t pool = nullptr;
  // Pinned host blocks by power-of-two size class, recycled across networks.
  std::multimap<size_t, void*> pinned_free;

  int dev_alloc(void** p, size_t bytes) {
    if (fail_alloc_after == 0) {
      fail_alloc_after = -1;
      return fail(CP_E_OOM, "device allocation of " + std::to_string(bytes) + " bytes: injected failure");
    }
    if (fail_alloc_after > 0) --fail_alloc_after;
    // Callers ask for 256 extra bytes to align the block's start themselves.
    cudaError_t err = cudaMallocFromPoolAsync(p, bytes, pool, stream);
    if (err != cudaSuccess) {
      cudaGetLastError();
      return fail(err == cudaErrorMemoryAllocation ? CP_E_OOM : CP_E_CUDA,
                  "device allocation of " + std::to_string(bytes) + " bytes: " + cudaGetErrorString(err));
    }
    return CP_OK;
  }
  void dev_free(void* p) {
    if (p) cudaFreeAsync(p, stream);
  }
  static size_t pinned_class(size_t bytes) {
    size_t c = 4096;
    while (c < bytes) c <<= 1;
    return c;
  }
  int pinned_get(size_t bytes, void** p) {
    const size_t c = pinned_class(bytes);
    auto it = pinned_free.find(c);
    if (it != pinned_free.end()) {
      *p = it->second;
      pinned_free.erase(it);
      return CP_OK;
    }
    cudaError_t err = cudaMallocHost(p, c);
    if (err != cudaSuccess) {
      cudaGetLastError();
      return fail(CP_E_OOM, std::string("pinned host allocation: ") + cudaGetErrorString(err));
    }
    return CP_OK;
  }
  void pinned_put(void* p, size_t bytes) {
    if (p) pinned_free.emplace(pinned_class(bytes), p);
  }
  int mapped_get(size_t bytes, void** p) {
    const size_t c = pinned_class(bytes);
    auto it = mapped_free.find(c);
    if (it != mapped_free.end()) {
      *p = it->second;
      mapped_free.erase(it);
      return CP_OK;
    }
    cudaError_t err = cudaHostAlloc(p, c, cudaHostAllocMapped);
    if (err != cudaSuccess) {
      cudaGetLastError();
      return fail(CP_E_OOM, std::string("mapped host allocation: ") + cudaGetErrorString(err));
    }
    return CP_OK;
  }
  void mapped_put(void* p, size_t bytes) {
    if (p) mapped_free.emplace(pinned_class(bytes), p);
  }
};

// Several host arrays packed at 256-byte offsets of one block.
struct MetaPack {
  struct Part {
    void** dst;
    const void* src;
    size_t bytes;
    size_t off;
  };
  std::vector<Part> parts;
  size_t total = 0;
  template <typename T>
  void add(T** dst, const T* src, size_t count) {
    const size_t bytes = count * sizeof(T);
    parts.push_back(Part{reinterpret_cast<void**>(dst), src, bytes, total});
    total += (std::max<size_t>(bytes, 16) + 255) & ~size_t(255);
  }
};

// A pinned host block borrowed from the engine for the duration of one call;
// the engine stream is drained before the block goes back, so copies that
// read from it have finished.
struct PinnedLease {
  cp_engine* e;
  void* p = nullptr;
  size_t bytes = 0;
  explicit PinnedLease(cp_engine* eng) : e(eng) {}
  int get(size_t n) {
    bytes = n;
    return e->pinned_get(n, &p);
  }
  ~PinnedLease() {
    if (p) {
      cudaStreamSynchronize(e->stream);
      e->pinned_put(p, bytes);
    }
  }
};

struct cp_net {
  cp_engine* e = nullptr;
  int n = 0, W_user = 1, W = 1, nb = 0, nt = 0, levels = 0;
  std::vector<int> dom;
  std::vector<int> nbr_count;  // distinct neighbour variables (Network::neighborhood sizes)
  std::vector<int> bx, by;
  DevNet dn;
  std::vector<void*> allocs;
  u64* d_levels = nullptr;
  u64* d_rel = nullptr;
  int* d_bx = nullptr;
  int* d_nbr = nullptr;  // nbr_count on the device (dom/deg in the device search)
  int* d_arc_con = nullptr;  // constraint id of every binary incidence (CSR order)
  // dom/wdeg: scratch of the sequential replay (allocated on first use).
  ReplayScratch replay{};
  u64* d_replay_dom = nullptr;
  uint8_t* d_replay_assigned = nullptr;
  int* d_replay_out = nullptr;
  int* d_by = nullptr;
  int64_t* d_offA = nullptr;
  int64_t* d_offB = nullptr;
  std::vector<int64_t> offA, offB;  // host copies: word offsets of each constraint's A / B rows
  int64_t relA_words = 0, relB_words = 0;
  int top = 0;                 // level stack top (cp_level_push / cp_level_pop_to)
  GridScratch G{};
  SacScratch S{};
  KStats* d_stats = nullptr;
  KStats* h_stats = nullptr;  // pinned
  int* d_evt = nullptr;       // n
  int* d_sizes = nullptr;     // n
  uint8_t* d_ok1 = nullptr;   // per-test results of the plain path
  u64* h_dom = nullptr;       // pinned n*W
  bool h_dom_pending = false; // an asynchronous reload may still be reading h_dom
  int* h_sizes = nullptr;     // pinned n
  void* d_cta_scratch = nullptr;  // k_node state when shared memory is too small
  void* d_sac_scratch = nullptr;
  size_t sac_stride = 0;
  int sac_grid = 0;
  int tile_grid = 0;   // persistent CTAs of the tiled sweep (0: not eligible)
  int slot_cap = 0;    // neighbours per tile held in shared memory
  int front_blocks = 0;  // cooperative grid of the whole-grid fixpoint
  bool cta_in_smem = true;
  bool prefer_grid = false;
  int64_t device_bytes = 0;
  int max_deg = 0;     // largest number of binary arcs at one variable

  void* h_block = nullptr;  // host-mapped pinned block holding h_stats, h_dom, h_sizes
  size_t h_block_bytes = 0;
  KStats* dh_stats = nullptr;  // device address of h_stats (written by k_stats_out)
  u64* dh_dom = nullptr;       // device address of h_dom (the last SAC commit writes the closure there)
  int sac_pending_level = -1;  // level of a SAC1 call begun and not yet ended
  int sac_pending_launches = 0;
  // SAC1 rounds captured as CUDA graphs: [0] root AC + sweep, [1] events AC +
  // sweep; valid for the level and knobs in sac_key.
  cudaGraphExec_t sac_exec[2] = {nullptr, nullptr};
  int sac_launches[2] = {0, 0};
  std::array<int64_t, 10> sac_key{};
  bool sac_graph_off = false;  // capture failed once: rounds run uncaptured

  void drop_sac_graphs() {
    for (auto& x : sac_exec) {
      if (x) cudaGraphExecDestroy(x);
      x = nullptr;
    }
  }

  ~cp_net() {
    drop_sac_graphs();
    if (e) {
      for (void* p : allocs) e->dev_free(p);
      e->mapped_put(h_block, h_block_bytes);
      --e->live_nets;
    }
  }

  // Allocations start on 256-byte boundaries (vector and bulk loads).
  template <typename T>
  int alloc(T** p, size_t count) {
    void* raw = nullptr;
    const size_t bytes = (std::max<size_t>(count * sizeof(T), 16) + 255) & ~size_t(255);
    CP_TRY(e->dev_alloc(&raw, bytes + 256));
    allocs.push_back(raw);
    device_bytes += static_cast<int64_t>(bytes);
    *p = reinterpret_cast<T*>((reinterpret_cast<uintptr_t>(raw) + 255) & ~uintptr_t(255));
    return CP_OK;
  }
  u64* level_ptr(int level) { return d_levels + static_cast<size_t>(level) * n * W; }
};

namespace {

// Device-to-host copy ordered after everything queued on the engine stream.
int d2h(cp_engine* e, void* dst, const void* src, size_t bytes) {
  if (bytes == 0) return CP_OK;
  CP_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, e->stream));
  CP_CUDA(cudaStreamSynchronize(e->stream));
  return CP_OK;
}

// ---- stats --------------------------------------------------------------
int stats_begin(cp_net* net) {
  KStats z{};
  z.fail_var = -1;
  *net->h_stats = z;
  CP_CUDA(cudaMemcpyAsync(net->d_stats, net->h_stats, sizeof(KStats), cudaMemcpyHostToDevice, net->e->stream));
  return CP_OK;
}

int stats_fetch(cp_net* net) {
  CP_CUDA(cudaMemcpyAsync(net->h_stats, net->d_stats, sizeof(KStats), cudaMemcpyDeviceToHost, net->e->stream));
  CP_CUDA(cudaStreamSynchronize(net->e->stream));
  if (net->h_stats->grid_err) return fail(CP_E_TIMEOUT, "device grid barrier wait ran out");
  if (net->h_stats->error) return fail(net->h_stats->error, "device-side check failed (round limit)");
  return CP_OK;
}

struct Acc {
  cp_stats s{};
  void add(const KStats& k, int launches) {
    s.revisions += static_cast<int64_t>(k.revisions);
    s.rows += static_cast<int64_t>(k.rows + k.tuples);
    s.fixpoints += static_cast<int64_t>(k.fixpoints);
    s.branches += static_cast<int64_t>(k.branches);
    s.rounds = std::max(s.rounds, k.rounds_max);
    s.launches += launches;
    tuples += static_cast<int64_t>(k.tuples);
    bin_rows += static_cast<int64_t>(k.rows);
    dels += static_cast<int64_t>(k.deletions);
  }
  int64_t tuples = 0, bin_rows = 0, dels = 0;
};

// Algorithmic bytes: support rows and tuples read, both domains of every
// revision read, changed words written, plus each SAC branch's domain copy.
double alg_bytes(const cp_net* net, const Acc& a, int64_t branches) {
  const double wb = 8.0 * net->W_user;
  return double(a.bin_rows) * wb + double(a.tuples) * 6.0 + double(a.s.revisions) * 2.0 * wb +
         double(a.dels) * wb + double(branches) * 2.0 * net->n * wb;
}

// ---- one AC fixpoint at a level ----------------------------------------
// evt_dev: device list of seeds (nullptr = all variables); nevt: its length.
// nevt_dev (optional, grid path only): the event count read on the device.
// ctl_cleared: the grid fixpoint's control block was already cleared (by
// k_round_prep) in stream order before this call.
int run_ac(cp_net* net, int level, const int* evt_dev, int nevt, int& launches, KStats* st = nullptr,
           const int* nevt_dev = nullptr, bool ctl_cleared = false) {
  cp_engine* e = net->e;
  if (!st) st = net->d_stats;
  if (net->prefer_grid) {
    cudaStream_t s = e->stream;
    if (!ctl_cleared)
      CP_CUDA(cudaMemsetAsync(net->G.flags, 0, net->G.ctl_words * sizeof(int), s));  // flags .. bitmaps
    net->G.wait_ns = e->wait_ns;
    CP_CUDA(launch_ac_front(net->dn, net->level_ptr(level), evt_dev, nevt_dev, evt_dev ? nevt : 0, net->G, st,
                            net->front_blocks, s));
    if (!evt_dev) {  // round 0 ran as its own launch
      ++launches;
      ++e->launches;
    }
  } else {
    const int op = evt_dev ? kOpEvents : kOpRoot;
    CP_CUDA(launch_node(net->dn, net->d_levels, level, level, op, 0, 0, evt_dev, nevt, st, nullptr,
                        e->block_node, net->cta_in_smem ? nullptr : net->d_cta_scratch, e->stream));
  }
  ++launches;
  ++e->launches;
  return CP_OK;
}

// Copies level `level` (internal width) to the pinned host mirror and
// converts to the user width into out (if given).
int fetch_level(cp_net* net, int level, uint64_t* out) {
  const size_t words = static_cast<size_t>(net->n) * net->W;
  CP_CUDA(cudaMemcpyAsync(net->h_dom, net->level_ptr(level), words * 8, cudaMemcpyDeviceToHost, net->e->stream));
  CP_CUDA(cudaStreamSynchronize(net->e->stream));
  if (out) {
    for (int x = 0; x < net->n; ++x)
      for (int w = 0; w < net->W_user; ++w)
        out[static_cast<size_t>(x) * net->W_user + w] = net->h_dom[static_cast<size_t>(x) * net->W + w];
  }
  return CP_OK;
}

int check_level(const cp_net* net, int level) {
  if (level < 0 || level >= net->levels) return fail(CP_E_ARG, "level out of range: " + std::to_string(level));
  return CP_OK;
}

int check_var_val(const cp_net* net, int var, int val) {
  if (var < 0 || var >= net->n) return fail(CP_E_ARG, "variable out of range: " + std::to_string(var));
  if (val < 0 || val >= net->dom[var]) return fail(CP_E_ARG, "value out of range: " + std::to_string(val));
  return CP_OK;
}

double elapsed_ms(cp_engine* e) {
  float ms = 0;
  cudaEventElapsedTime(&ms, e->ev0, e->ev1);
  return ms;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* cp_last_error_string(void) { return g_last_error.c_str(); }

int cp_engine_create(int device, cp_engine** out) {
  if (!out) return fail(CP_E_ARG, "null output pointer");
  int count = 0;
  CP_CUDA(cudaGetDeviceCount(&count));
  if (device < 0 || device >= count) return fail(CP_E_ARG, "no CUDA device " + std::to_string(device));
  CP_CUDA(cudaSetDevice(device));
  auto e = std::make_unique<cp_engine>();
  e->device = device;
  cudaDeviceProp prop;
  CP_CUDA(cudaGetDeviceProperties(&prop, device));
  if (!prop.cooperativeLaunch) return fail(CP_E_UNSUPPORTED, "device lacks cooperative launch");
  e->sm_count = prop.multiProcessorCount;
  e->smem_optin = prop.sharedMemPerBlockOptin;
  CP_CUDA(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking));
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  CP_CUDA(cudaMemPoolCreate(&e->pool, &props));
  uint64_t keep = UINT64_MAX;  // freed blocks stay in the pool for the next network
  CP_CUDA(cudaMemPoolSetAttribute(e->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  CP_CUDA(cudaEventCreate(&e->ev0));
  CP_CUDA(cudaEventCreate(&e->ev1));
  CP_CUDA(cudaEventCreate(&e->evk0));
  CP_CUDA(cudaEventCreate(&e->evk1));
  *out = e.release();
  return CP_OK;
}

// An engine outlives its networks: destroying it while networks are alive
// only marks it closed, and the last network destroyed frees it.
static void engine_free(cp_engine* e) {
  cudaSetDevice(e->device);
  if (e->stream) cudaStreamSynchronize(e->stream);
  for (auto& kv : e->pinned_free) cudaFreeHost(kv.second);
  for (auto& kv : e->mapped_free) cudaFreeHost(kv.second);
  if (e->pool) cudaMemPoolDestroy(e->pool);
  if (e->ev0) cudaEventDestroy(e->ev0);
  if (e->ev1) cudaEventDestroy(e->ev1);
  if (e->evk0) cudaEventDestroy(e->evk0);
  if (e->evk1) cudaEventDestroy(e->evk1);
  if (e->xfer) {
    cudaStreamSynchronize(e->xfer);
    cudaStreamDestroy(e->xfer);
  }
  if (e->xfer_ev) cudaEventDestroy(e->xfer_ev);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

int cp_engine_destroy(cp_engine* e) {
  if (!e) return CP_OK;
  if (e->closed) return fail(CP_E_STATE, "engine destroyed twice");
  e->closed = true;
  if (e->live_nets == 0) engine_free(e);
  return CP_OK;
}

int64_t cp_engine_launches(const cp_engine* e) { return e ? e->launches : 0; }
int cp_engine_device(const cp_engine* e) { return e ? e->device : -1; }

int cp_engine_set_tuning(cp_engine* e, int block, int chunk, int ctas_per_sm) {
  if (!e) return fail(CP_E_ARG, "null engine");
  if (block < 0 || block > 1024 || (block % 32) != 0) return fail(CP_E_ARG, "block must be a multiple of 32 <= 1024");
  if (block) {
    e->block_node = block;
    e->block_sac = std::min(block, 256);
  }
  e->chunk = chunk;
  e->ctas_per_sm = ctas_per_sm;
  return CP_OK;
}

int cp_engine_set_sac_mode(cp_engine* e, int mode) {
  if (!e) return fail(CP_E_ARG, "null engine");
  if (mode != 0 && mode != 1) return fail(CP_E_ARG, "SAC mode must be 0 (tiled where eligible) or 1 (general)");
  e->sac_mode = mode;
  return CP_OK;
}

int cp_engine_set_graphs(cp_engine* e, int use_graphs) {
  if (!e) return fail(CP_E_ARG, "null engine");
  e->sac_graphs = use_graphs != 0;
  return CP_OK;
}

int cp_engine_set_priority(cp_engine* e, int priority) {
  if (!e) return fail(CP_E_ARG, "null engine");
  if (priority < -1 || priority > 1) return fail(CP_E_ARG, "priority must be -1, 0 or 1");
  if (e->live_nets > 0) return fail(CP_E_STATE, "stream priority is set before any network is uploaded");
  CP_CUDA(cudaSetDevice(e->device));
  int least = 0, greatest = 0;
  CP_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  const int p = priority > 0 ? greatest : (priority < 0 ? least : 0);
  cudaStream_t ns = nullptr;
  CP_CUDA(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, p));
  CP_CUDA(cudaStreamSynchronize(e->stream));
  CP_CUDA(cudaStreamDestroy(e->stream));
  e->stream = ns;
  e->priority = priority;
  return CP_OK;
}

int cp_engine_set_wait_budget(cp_engine* e, int64_t ns) {
  if (!e) return fail(CP_E_ARG, "null engine");
  if (ns < 0) return fail(CP_E_ARG, "negative wait budget");
  e->wait_ns = ns;
  return CP_OK;
}

int cp_engine_inject_alloc_failure(cp_engine* e, int64_t after) {
  if (!e) return fail(CP_E_ARG, "null engine");
  if (after < -1) return fail(CP_E_ARG, "after must be -1 (off) or >= 0");
  e->fail_alloc_after = after;
  return CP_OK;
}

int cp_engine_set_cta_quota(cp_engine* e, int quota) {
  if (!e) return fail(CP_E_ARG, "null engine");
  if (quota < 0) return fail(CP_E_ARG, "negative quota");
  e->cta_quota = quota;
  return CP_OK;
}

// rows_later: the binary rows are filled afterwards on the device (seeded
// generator), so bin_rows may be null.
static int net_upload_impl(cp_engine* e, int n, const int* dom, int W, const uint64_t* init, int n_bin,
                           const int* bin_scope, const uint64_t* bin_rows, int n_tab, const int* tab_arity,
                           const int* tab_scope, const int* tab_ntup, const int* tab_tuples, int max_levels,
                           cp_net** out, bool rows_later) {
  if (!e || !out) return fail(CP_E_ARG, "null engine or output");
  if (n < 1 || n >= kMaxVars) return fail(CP_E_ARG, "n out of range");
  if (!dom || !init) return fail(CP_E_ARG, "null dom or init");
  if (n_bin < 0 || n_tab < 0) return fail(CP_E_ARG, "negative constraint count");
  if (n_bin > 0 && (!bin_scope || (!bin_rows && !rows_later))) return fail(CP_E_ARG, "null binary arrays");
  if (n_tab > 0 && (!tab_arity || !tab_scope || !tab_ntup || !tab_tuples)) return fail(CP_E_ARG, "null table arrays");
  const int Wi = internal_words(W);
  if (W < 1 || Wi < 0) return fail(CP_E_UNSUPPORTED, "domains wider than 512 values are not supported");
  for (int x = 0; x < n; ++x)
    if (dom[x] < 1 || dom[x] > 64 * W) return fail(CP_E_ARG, "domain size of variable " + std::to_string(x));
  CP_CUDA(cudaSetDevice(e->device));
  auto net = std::make_unique<cp_net>();
  net->e = e;
  ++e->live_nets;
  net->n = n;
  net->W_user = W;
  net->W = Wi;
  net->nb = n_bin;
  net->nt = n_tab;
  net->dom.assign(dom, dom + n);
  net->levels = max_levels > 0 ? max_levels : n + 3;
  if (net->levels < 2) net->levels = 2;

  // Binary constraints: scopes, relation offsets, arcs by source variable.
  net->bx.resize(n_bin);
  net->by.resize(n_bin);
  std::vector<int64_t> offA(n_bin), offB(n_bin);
  int64_t ta = 0, tb = 0;
  std::vector<int> arc_deg(n, 0), tab_deg(n, 0);
  for (int c = 0; c < n_bin; ++c) {
    const int x = bin_scope[2 * c], y = bin_scope[2 * c + 1];
    if (x < 0 || x >= n || y < 0 || y >= n || x == y) return fail(CP_E_ARG, "bad binary scope " + std::to_string(c));
    net->bx[c] = x;
    net->by[c] = y;
    offA[c] = ta;
    ta += static_cast<int64_t>(dom[x]) * Wi;
    ++arc_deg[x];
    ++arc_deg[y];
  }
  for (int c = 0; c < n_bin; ++c) {
    offB[c] = ta + tb;
    tb += static_cast<int64_t>(net->dom[net->by[c]]) * Wi;
  }
  if (ta + tb >= (int64_t(1) << 32)) return fail(CP_E_UNSUPPORTED, "relations exceed 32 GiB");
  net->relA_words = ta;
  net->relB_words = tb;
  std::vector<int> arc_start(n + 1, 0);
  for (int x = 0; x < n; ++x) arc_start[x + 1] = arc_start[x] + arc_deg[x];
  std::vector<Arc> arcs(static_cast<size_t>(2) * n_bin);
  std::vector<int> arc_con(static_cast<size_t>(2) * n_bin);
  {
    // One pass over the constraints in order: every variable's incidences are
    // in increasing constraint order (the reference's subscription order).
    std::vector<int> fill(arc_start.begin(), arc_start.end() - 1);
    for (int c = 0; c < n_bin; ++c) {
      const int x = net->bx[c], y = net->by[c];
      // Source y: revise x against y (x's rows are the A block).
      arc_con[fill[y]] = c;
      arcs[fill[y]++] = Arc{x, static_cast<u32>(offA[c]), static_cast<u32>(offB[c]), y};
      // Source x: revise y against x (y's rows are the B block).
      arc_con[fill[x]] = c;
      arcs[fill[x]++] = Arc{y, static_cast<u32>(offB[c]), static_cast<u32>(offA[c]), x};
    }
  }
  // Tables.
  std::vector<int> t_arity(n_tab), t_soff(n_tab), t_scope, t_ntup(n_tab);
  std::vector<int> t_scope4(static_cast<size_t>(n_tab) * kMaxArity, 0);
  std::vector<int64_t> t_off(n_tab);
  int64_t total_tup = 0;
  {
    int64_t so = 0;
    std::vector<int> seen(n, -1);
    for (int t = 0; t < n_tab; ++t) {
      const int r = tab_arity[t];
      if (r < 2 || r > n) return fail(CP_E_ARG, "table arity must be 2..n");
      if (tab_ntup[t] < 0) return fail(CP_E_ARG, "negative tuple count");
      t_arity[t] = r;
      t_soff[t] = static_cast<int>(t_scope.size());
      for (int i = 0; i < r; ++i) {
        const int v = tab_scope[so + i];
        if (v < 0 || v >= n) return fail(CP_E_ARG, "bad table scope " + std::to_string(t));
        if (seen[v] == t) return fail(CP_E_ARG, "repeated variable in table");
        seen[v] = t;
        t_scope.push_back(v);
        if (i < kMaxArity) t_scope4[static_cast<size_t>(t) * kMaxArity + i] = v;
        ++tab_deg[v];
      }
      so += r;
      t_ntup[t] = tab_ntup[t];
      t_off[t] = total_tup;
      total_tup += static_cast<int64_t>(tab_ntup[t]) * r;
    }
    if (so > INT32_MAX) return fail(CP_E_UNSUPPORTED, "table scopes too long");
  }
  std::vector<uint16_t> t_tup(static_cast<size_t>(total_tup));
  {
    int64_t src = 0;
    for (int t = 0; t < n_tab; ++t) {
      const int r = t_arity[t], k = t_ntup[t];
      for (int j = 0; j < k; ++j)
        for (int i = 0; i < r; ++i) {
          const int v = tab_tuples[src + static_cast<int64_t>(j) * r + i];
          const int var = t_scope[t_soff[t] + i];
          if (v < 0 || v >= dom[var]) return fail(CP_E_ARG, "tuple value out of range in table " + std::to_string(t));
          t_tup[t_off[t] + static_cast<int64_t>(i) * k + j] = static_cast<uint16_t>(v);
        }
      src += static_cast<int64_t>(k) * r;
    }
  }
  {
    // Network::get_neighbor (src/Network.cpp:467-476): the distinct other
    // variables of every constraint on x; the dom/deg variable order divides
    // by their number.
    std::vector<std::vector<int>> adj(n);
    for (int c = 0; c < n_bin; ++c) {
      adj[net->bx[c]].push_back(net->by[c]);
      adj[net->by[c]].push_back(net->bx[c]);
    }
    for (int t = 0; t < n_tab; ++t)
      for (int i = 0; i < t_arity[t]; ++i)
        for (int j = 0; j < t_arity[t]; ++j)
          if (i != j)
            adj[t_scope[t_soff[t] + i]].push_back(t_scope[t_soff[t] + j]);
    net->nbr_count.resize(n);
    for (int x = 0; x < n; ++x) {
      std::sort(adj[x].begin(), adj[x].end());
      net->nbr_count[x] = static_cast<int>(std::unique(adj[x].begin(), adj[x].end()) - adj[x].begin());
    }
  }
  std::vector<int> tinc_start(n + 1, 0);
  for (int x = 0; x < n; ++x) tinc_start[x + 1] = tinc_start[x] + tab_deg[x];
  std::vector<int> vtab(tinc_start[n]);
  {
    std::vector<int> fill(tinc_start.begin(), tinc_start.end() - 1);
    for (int t = 0; t < n_tab; ++t)
      for (int i = 0; i < t_arity[t]; ++i) vtab[fill[t_scope[t_soff[t] + i]]++] = t;
  }
  // Work-item chunking.
  const int chunk = e->chunk > 0 ? e->chunk : 8;
  int64_t total_values = 0;
  for (int x = 0; x < n; ++x) total_values += dom[x];

  // Device allocations and copies.
  cudaStream_t s = e->stream;
  DevNet& D = net->dn;
  D.n = n;
  D.W = Wi;
  D.nb = n_bin;
  D.nt = n_tab;
  D.chunk = chunk;
  D.total_values = total_values;
  int* d_dsize;
  int* d_arc_start;
  Arc* d_arcs;
  int* d_tinc;
  int* d_vtab;
  int *d_tar, *d_tsc, *d_tso, *d_ts4, *d_tnt;
  int64_t* d_toff;
  uint16_t* d_ttup;
  // Metadata arrays: one device block, filled by one copy from pinned staging.
  MetaPack mp;
  mp.add(&d_dsize, dom, n);
  mp.add(&d_arc_start, arc_start.data(), n + 1);
  mp.add(&d_arcs, arcs.data(), arcs.size());
  mp.add(&d_tinc, tinc_start.data(), n + 1);
  mp.add(&d_vtab, vtab.data(), vtab.size());
  mp.add(&d_tar, t_arity.data(), n_tab);
  mp.add(&d_tsc, t_scope.data(), t_scope.size());
  mp.add(&d_tso, t_soff.data(), n_tab);
  mp.add(&d_ts4, t_scope4.data(), t_scope4.size());
  mp.add(&d_tnt, t_ntup.data(), n_tab);
  mp.add(&d_toff, t_off.data(), n_tab);
  mp.add(&d_ttup, t_tup.data(), t_tup.size());
  mp.add(&net->d_bx, net->bx.data(), n_bin);
  mp.add(&net->d_nbr, net->nbr_count.data(), n);
  mp.add(&net->d_arc_con, arc_con.data(), arc_con.size());
  mp.add(&net->d_by, net->by.data(), n_bin);
  mp.add(&net->d_offA, offA.data(), n_bin);
  mp.add(&net->d_offB, offB.data(), n_bin);
  net->offA = offA;
  net->offB = offB;
  char* d_meta = nullptr;
  CP_TRY(net->alloc(&d_meta, mp.total));
  PinnedLease stage(e);
  CP_TRY(stage.get(mp.total));
  for (const auto& q : mp.parts) {
    if (q.bytes) std::memcpy(static_cast<char*>(stage.p) + q.off, q.src, q.bytes);
    *q.dst = d_meta + q.off;
  }
  CP_CUDA(cudaMemcpyAsync(d_meta, stage.p, mp.total, cudaMemcpyHostToDevice, s));
  CP_TRY(net->alloc(&net->d_rel, static_cast<size_t>(ta + tb)));
  CP_TRY(net->alloc(&net->d_levels, static_cast<size_t>(net->levels) * n * Wi));
  D.dsize = d_dsize;
  D.arc_start = d_arc_start;
  D.arcs = d_arcs;
  D.tinc_start = d_tinc;
  D.vtab = d_vtab;
  D.rel = net->d_rel;
  D.t_arity = d_tar;
  D.t_scope = d_tsc;
  D.t_soff = d_tso;
  D.t_scope4 = d_ts4;
  D.t_ntup = d_tnt;
  D.t_off = d_toff;
  D.t_tup = d_ttup;

  // Scratch.
  const size_t nw = (static_cast<size_t>(n) + 31) / 32;
  GridScratch& G = net->G;
  {
    // flags[3] + pad | failed[2] + pad | bar[2] + pad | three bitmaps:
    // cleared by one memset before each launch.
    G.ctl_words = 12 + 3 * nw;
    int* ctl;
    CP_TRY(net->alloc(&ctl, G.ctl_words));
    G.flags = ctl;
    G.failed = ctl + 4;
    G.bar = reinterpret_cast<unsigned*>(ctl + 8);
    G.bm = reinterpret_cast<u32*>(ctl + 12);
  }
  SacScratch& S = net->S;
  CP_TRY(net->alloc(&S.work, total_values));
  CP_TRY(net->alloc(&S.ok, total_values));
  CP_TRY(net->alloc(&S.evt, n));
  CP_TRY(net->alloc(&S.evt_fb, nw));
  CP_TRY(net->alloc(&S.tiles, static_cast<size_t>(n) * 2 * Wi));
  CP_TRY(net->alloc(&S.deep, total_values));
  // The sweep counters sit together so that one memset clears them.
  int* ctr = nullptr;
  CP_TRY(net->alloc(&ctr, 8));  // [7]: k_commit's completion counter, zero between launches
  CP_CUDA(cudaMemsetAsync(ctr, 0, 8 * sizeof(int), e->stream));
  S.nwork = ctr;
  S.cursor = ctr + 1;
  S.nevt = ctr + 2;
  S.ntiles = ctr + 3;
  S.tcursor = ctr + 4;
  S.ndeep = ctr + 5;
  S.weak = nullptr;
  if (n_tab == 0 && n_bin > 0) CP_TRY(net->alloc(&S.weak, static_cast<size_t>(2) * n_bin * kWeakStride));
  CP_TRY(net->alloc(&S.snap, static_cast<size_t>(n) * Wi));
  CP_TRY(net->alloc(&net->d_stats, 2));  // [0] the call's kernels, [1] a level AC queued without a sync
  CP_TRY(net->alloc(&net->d_evt, n));
  CP_TRY(net->alloc(&net->d_sizes, n));
  CP_TRY(net->alloc(&net->d_ok1, total_values));
  {
    static_assert(2 * sizeof(KStats) <= 512, "two stats slots in the pinned block");
    const size_t st_bytes = 512;  // the two stats slots fetched after each call
    const size_t dom_bytes = (static_cast<size_t>(n) * Wi * 8 + 255) & ~size_t(255);
    net->h_block_bytes = st_bytes + dom_bytes + static_cast<size_t>(n) * sizeof(int);
    CP_TRY(e->mapped_get(net->h_block_bytes, &net->h_block));
    char* hb = static_cast<char*>(net->h_block);
    net->h_stats = reinterpret_cast<KStats*>(hb);
    {
      void* dh = nullptr;
      CP_CUDA(cudaHostGetDevicePointer(&dh, net->h_block, 0));
      net->dh_stats = static_cast<KStats*>(dh);
      net->dh_dom = reinterpret_cast<u64*>(static_cast<char*>(dh) + st_bytes);
    }
    net->h_dom = reinterpret_cast<u64*>(hb + st_bytes);
    net->h_sizes = reinterpret_cast<int*>(hb + st_bytes + dom_bytes);
  }

  // CTA-local state: shared memory when it fits, else global scratch.
  const size_t cta_bytes = cta_state_bytes(D);
  net->cta_in_smem = cta_bytes + 1024 <= e->smem_optin;
  if (!net->cta_in_smem) {
    char* p;
    CP_TRY(net->alloc(&p, cta_bytes));
    net->d_cta_scratch = p;
  }
  // Persistent SAC grid.
  int per_sm = sac_blocks_per_sm(D, e->block_sac, net->cta_in_smem);
  if (per_sm < 1) return fail(CP_E_UNSUPPORTED, "SAC kernel does not fit on an SM");
  if (e->ctas_per_sm > 0) per_sm = std::min(per_sm, e->ctas_per_sm);
  net->sac_grid = per_sm * e->sm_count;
  if (!net->cta_in_smem) {
    net->sac_stride = (cta_bytes + 255) & ~size_t(255);
    char* p;
    CP_TRY(net->alloc(&p, net->sac_stride * net->sac_grid));
    net->d_sac_scratch = p;
  }
  net->front_blocks = ac_front_blocks(D, static_cast<int>(arcs.size()), e->sm_count);
  if (net->front_blocks < 1) return fail(CP_E_UNSUPPORTED, "grid fixpoint kernel does not fit");
  // Tiled SAC sweep (binary networks): shared memory holds the round-one
  // domains of up to slot_cap neighbours for 32 branches, plus a slot map.
  for (int x = 0; x < n; ++x) net->max_deg = std::max(net->max_deg, arc_deg[x]);
  if (n_tab == 0) {
    const size_t per_slot = static_cast<size_t>(32) * Wi * 8 + 16;  // domains + neighbour record
    int cap = std::max(net->max_deg, 1);
    // 100 KB keeps two or more tile CTAs per SM; a network whose densest
    // variable needs more gets up to the opt-in limit (fewer, larger CTAs)
    // rather than sending those variables' branches to the general kernel.
    const size_t optin = e->smem_optin > 4096 ? e->smem_optin - 4096 : 0;
    const size_t need = static_cast<size_t>(n) * 4 + per_slot * static_cast<size_t>(cap);
    const size_t budget = std::min<size_t>(optin, std::max<size_t>(100 * 1024, need));
    if (static_cast<size_t>(n) * 4 + per_slot * 8 <= budget) {
      const size_t fit = (budget - static_cast<size_t>(n) * 4) / per_slot;
      net->slot_cap = static_cast<int>(std::min<size_t>(static_cast<size_t>(cap), fit));
      const int per_sm_t = sac_tile_blocks_per_sm(D, net->slot_cap, kTileBlock);
      net->tile_grid = per_sm_t > 0 ? per_sm_t * e->sm_count : 0;
    }
  }
  // Large networks run their single-instance fixpoints on the whole grid.
  net->prefer_grid = (2 * static_cast<int64_t>(n_bin) + n_tab) > 8192 || !net->cta_in_smem;

  // Relations: A blocks from the user's rows, B blocks transposed on device.
  CP_TRY(cp_net_reload(net.get(), init, bin_rows));
  *out = net.release();
  return CP_OK;
}

int cp_net_upload(cp_engine* e, int n, const int* dom, int W, const uint64_t* init, int n_bin, const int* bin_scope,
                  const uint64_t* bin_rows, int n_tab, const int* tab_arity, const int* tab_scope,
                  const int* tab_ntup, const int* tab_tuples, int max_levels, cp_net** out) {
  return net_upload_impl(e, n, dom, W, init, n_bin, bin_scope, bin_rows, n_tab, tab_arity, tab_scope, tab_ntup,
                         tab_tuples, max_levels, out, false);
}

// Waits for an asynchronous reload's copy out of h_dom before the host
// writes h_dom again.
static int settle_h_dom(cp_net* net) {
  if (net->h_dom_pending) {
    CP_CUDA(cudaStreamSynchronize(net->e->xfer));
    net->h_dom_pending = false;
  }
  return CP_OK;
}

static int net_reload_impl(cp_net* net, const uint64_t* init, const uint64_t* bin_rows, bool wait) {
  if (!net) return fail(CP_E_ARG, "null net");
  cp_engine* e = net->e;
  CP_TRY(settle_h_dom(net));
  if (!wait && !e->xfer) {
    int least = 0, greatest = 0;
    CP_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CP_CUDA(cudaStreamCreateWithPriority(&e->xfer, cudaStreamNonBlocking, least));
    CP_CUDA(cudaEventCreateWithFlags(&e->xfer_ev, cudaEventDisableTiming));
  }
  // The asynchronous form queues behind the engine's earlier work.
  if (!wait) {
    CP_CUDA(cudaEventRecord(e->xfer_ev, e->stream));
    CP_CUDA(cudaStreamWaitEvent(e->xfer, e->xfer_ev, 0));
  }
  cudaStream_t s = wait ? e->stream : e->xfer;
  const int W = net->W_user, Wi = net->W, n = net->n;
  if (net->nb > 0 && bin_rows) {
    if (W == Wi) {
      CP_CUDA(cudaMemcpyAsync(net->d_rel, bin_rows, static_cast<size_t>(net->relA_words) * 8, cudaMemcpyHostToDevice, s));
    } else {
      std::vector<u64> pad(static_cast<size_t>(net->relA_words), 0);
      int64_t src = 0, dst = 0;
      for (int c = 0; c < net->nb; ++c)
        for (int a = 0; a < net->dom[net->bx[c]]; ++a) {
          for (int w = 0; w < W; ++w) pad[dst + w] = bin_rows[src + w];
          src += W;
          dst += Wi;
        }
      CP_CUDA(cudaMemcpyAsync(net->d_rel, pad.data(), pad.size() * 8, cudaMemcpyHostToDevice, s));
      CP_CUDA(cudaStreamSynchronize(s));
    }
    // k_transpose writes every word of the B blocks (dom[y] rows each).
    CP_CUDA(launch_transpose(net->dn, net->d_rel, net->d_bx, net->d_by, net->d_offA, net->d_offB, s));
    ++e->launches;
  }
  if (init) {
    // Bits at or beyond a variable's size are cleared: the kernels index
    // support rows by live values, so a stray bit would read past the block.
    for (int x = 0; x < n; ++x)
      for (int w = 0; w < Wi; ++w) {
        u64 v = w < W ? init[static_cast<size_t>(x) * W + w] : 0ull;
        const int lo = w * 64, d = net->dom[x];
        if (d - lo < 64) v &= (d - lo <= 0) ? 0ull : ((1ull << (d - lo)) - 1ull);
        net->h_dom[static_cast<size_t>(x) * Wi + w] = v;
      }
    CP_CUDA(cudaMemcpyAsync(net->d_levels, net->h_dom, static_cast<size_t>(n) * Wi * 8, cudaMemcpyHostToDevice, s));
  }
  if (wait) {
    CP_CUDA(cudaStreamSynchronize(s));
  } else {
    CP_CUDA(cudaEventRecord(e->xfer_ev, s));
    CP_CUDA(cudaStreamWaitEvent(e->stream, e->xfer_ev, 0));
    net->h_dom_pending = init != nullptr;
  }
  return CP_OK;
}

int cp_net_reload(cp_net* net, const uint64_t* init, const uint64_t* bin_rows) {
  return net_reload_impl(net, init, bin_rows, true);
}

int cp_net_reload_async(cp_net* net, const uint64_t* init, const uint64_t* bin_rows) {
  return net_reload_impl(net, init, bin_rows, false);
}

int cp_net_destroy(cp_net* net) {
  if (!net) return CP_OK;
  cp_engine* e = net->e;
  cudaSetDevice(e->device);
  cudaStreamSynchronize(e->stream);
  delete net;  // ~cp_net releases its hold on the engine
  if (e->closed && e->live_nets == 0) engine_free(e);
  return CP_OK;
}

int64_t cp_net_device_bytes(const cp_net* net) { return net ? net->device_bytes : 0; }

int cp_level_copy(cp_net* net, int src, int dst) {
  if (!net) return fail(CP_E_ARG, "null net");
  CP_TRY(check_level(net, src));
  CP_TRY(check_level(net, dst));
  if (src == dst) return CP_OK;
  const size_t bytes = static_cast<size_t>(net->n) * net->W * 8;
  CP_CUDA(cudaMemcpyAsync(net->level_ptr(dst), net->level_ptr(src), bytes, cudaMemcpyDeviceToDevice, net->e->stream));
  CP_CUDA(cudaStreamSynchronize(net->e->stream));
  return CP_OK;
}

int cp_dom_get(cp_net* net, int level, uint64_t* out) {
  if (!net || !out) return fail(CP_E_ARG, "null argument");
  CP_TRY(check_level(net, level));
  return fetch_level(net, level, out);
}

int cp_dom_set(cp_net* net, int level, const uint64_t* in) {
  if (!net || !in) return fail(CP_E_ARG, "null argument");
  CP_TRY(check_level(net, level));
  CP_TRY(settle_h_dom(net));
  const int W = net->W_user, Wi = net->W;
  for (int x = 0; x < net->n; ++x)
    for (int w = 0; w < Wi; ++w) {
      u64 v = w < W ? in[static_cast<size_t>(x) * W + w] : 0ull;
      const int lo = w * 64, d = net->dom[x];
      if (d - lo < 64) v &= (d - lo <= 0) ? 0ull : ((1ull << (d - lo)) - 1ull);
      net->h_dom[static_cast<size_t>(x) * Wi + w] = v;
    }
  CP_CUDA(cudaMemcpyAsync(net->level_ptr(level), net->h_dom, static_cast<size_t>(net->n) * Wi * 8,
                          cudaMemcpyHostToDevice, net->e->stream));
  CP_CUDA(cudaStreamSynchronize(net->e->stream));
  return CP_OK;
}

int cp_dom_sizes(cp_net* net, int level, int* out) {
  if (!net || !out) return fail(CP_E_ARG, "null argument");
  CP_TRY(check_level(net, level));
  CP_CUDA(launch_popcount(net->dn, net->level_ptr(level), net->d_sizes, net->e->stream));
  ++net->e->launches;
  CP_CUDA(cudaMemcpyAsync(out, net->d_sizes, net->n * sizeof(int), cudaMemcpyDeviceToHost, net->e->stream));
  CP_CUDA(cudaStreamSynchronize(net->e->stream));
  return CP_OK;
}

int cp_reduce_to(cp_net* net, int level, int var, int value) {
  if (!net) return fail(CP_E_ARG, "null net");
  CP_TRY(check_level(net, level));
  CP_TRY(check_var_val(net, var, value));
  CP_CUDA(launch_level_edit(net->dn, net->level_ptr(level), var, value, kOpAssign, net->e->stream));
  ++net->e->launches;
  CP_CUDA(cudaStreamSynchronize(net->e->stream));
  return CP_OK;
}

int cp_level_push(cp_net* net, int src, int* new_level) {
  if (!net || !new_level) return fail(CP_E_ARG, "null argument");
  CP_TRY(check_level(net, src));
  CP_TRY(check_level(net, src + 1));
  CP_TRY(cp_level_copy(net, src, src + 1));
  net->top = src + 1;
  *new_level = src + 1;
  return CP_OK;
}

int cp_level_pop_to(cp_net* net, int level) {
  if (!net) return fail(CP_E_ARG, "null net");
  CP_TRY(check_level(net, level));
  net->top = level;
  return CP_OK;
}

int cp_level_top(const cp_net* net) { return net ? net->top : CP_E_ARG; }

int cp_dom_set_var(cp_net* net, int level, int var, const uint64_t* words) {
  if (!net || !words) return fail(CP_E_ARG, "null argument");
  CP_TRY(check_level(net, level));
  if (var < 0 || var >= net->n) return fail(CP_E_ARG, "variable out of range");
  const int W = net->W_user, Wi = net->W, d = net->dom[var];
  u64 v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int w = 0; w < Wi; ++w) {
    u64 x = w < W ? words[w] : 0ull;
    const int lo = w * 64;
    if (d - lo < 64) x &= (d - lo <= 0) ? 0ull : ((1ull << (d - lo)) - 1ull);
    v[w] = x;
  }
  CP_CUDA(cudaMemcpyAsync(net->level_ptr(level) + static_cast<size_t>(var) * Wi, v, static_cast<size_t>(Wi) * 8,
                          cudaMemcpyHostToDevice, net->e->stream));
  CP_CUDA(cudaStreamSynchronize(net->e->stream));
  return CP_OK;
}

int cp_remove(cp_net* net, int level, int var, int value) {
  if (!net) return fail(CP_E_ARG, "null net");
  CP_TRY(check_level(net, level));
  CP_TRY(check_var_val(net, var, value));
  CP_CUDA(launch_level_edit(net->dn, net->level_ptr(level), var, value, kOpRefute, net->e->stream));
  ++net->e->launches;
  CP_CUDA(cudaStreamSynchronize(net->e->stream));
  return CP_OK;
}

int cp_enforce_ac(cp_net* net, int level, int n_evt, const int* evt, cp_stats* st) {
  if (!net) return fail(CP_E_ARG, "null net");
  CP_TRY(check_level(net, level));
  cp_engine* e = net->e;
  const int* evt_dev = nullptr;
  if (evt && n_evt > 0) {
    if (n_evt > net->n) return fail(CP_E_ARG, "too many event variables");
    for (int i = 0; i < n_evt; ++i)
      if (evt[i] < 0 || evt[i] >= net->n) return fail(CP_E_ARG, "event variable out of range");
    std::memcpy(net->h_sizes, evt, n_evt * sizeof(int));
    CP_CUDA(cudaMemcpyAsync(net->d_evt, net->h_sizes, n_evt * sizeof(int), cudaMemcpyHostToDevice, e->stream));
    evt_dev = net->d_evt;
  }
  CP_TRY(stats_begin(net));
  CP_CUDA(cudaEventRecord(e->ev0, e->stream));
  int launches = 0;
  CP_TRY(run_ac(net, level, evt_dev, evt_dev ? n_evt : 0, launches));
  CP_CUDA(cudaEventRecord(e->ev1, e->stream));
  CP_TRY(stats_fetch(net));
  if (st) {
    Acc a;
    a.add(*net->h_stats, launches);
    a.s.inconsistent = net->h_stats->inconsistent;
    a.s.deletions = a.dels;
    a.s.device_ms = elapsed_ms(e);
    a.s.alg_bytes = alg_bytes(net, a, 0);
    *st = a.s;
  }
  return CP_OK;
}

}  // extern "C"

namespace {

// One SAC1 round on the engine stream: both stats slots reset, the level AC
// into slot 1 (the root AC, SAC1::enforce src/SAC1.cpp:58, or the AC of the
// previous commit's removals, :85-92), then one sweep into slot 0, then both
// slots copied to the pinned mirror. Nothing waits on the host, except the
// events AC of a network without the grid path, which reads the event count
// first. A sweep queued behind an AC that wiped a domain out only wastes its
// work; its results are not used.
// sweep_only: a Jacobi sweep that removes nothing (no early removals, no
// commit), for cp_sac_sweep.
int sac_round_launches(cp_net* net, int level, bool root, int& launches, bool captured, bool sweep_only = false) {
  cp_engine* e = net->e;
  cudaStream_t s = e->stream;
  // Kernel-time events: external records become event nodes of a captured round.
  const unsigned evf = captured ? cudaEventRecordExternal : cudaEventRecordDefault;
  // Stats slots and (grid fixpoint) control block in one kernel.
  CP_CUDA(launch_round_prep(net->d_stats, net->prefer_grid ? net->G.flags : nullptr,
                            net->prefer_grid ? net->G.ctl_words : 0, s));
  if (root) {
    CP_TRY(run_ac(net, level, nullptr, 0, launches, net->d_stats + 1, nullptr, true));
  } else if (net->prefer_grid) {
    CP_TRY(run_ac(net, level, net->S.evt, 0, launches, net->d_stats + 1, net->S.nevt, true));
  } else {
    CP_CUDA(cudaMemcpyAsync(&net->h_sizes[0], net->S.nevt, sizeof(int), cudaMemcpyDeviceToHost, s));
    CP_CUDA(cudaStreamSynchronize(s));
    CP_TRY(run_ac(net, level, net->S.evt, net->h_sizes[0], launches, net->d_stats + 1));
  }
  const size_t nw = (static_cast<size_t>(net->n) + 31) / 32;
  CP_CUDA(launch_round_clear(net->S.nwork, 6, net->S.evt_fb, static_cast<int>(nw), s));  // nwork .. ndeep
  const bool tiled = net->tile_grid > 0 && e->sac_mode == 0;
  SacScratch S = net->S;
  if (!tiled) S.tiles = nullptr;
  launches += 2;
  e->launches += 2;
  const bool with_weak = tiled && S.weak;
  if (!with_weak) CP_CUDA(launch_build_work(net->dn, net->level_ptr(level), S, tiled ? S.snap : nullptr, s));
  CP_CUDA(cudaEventRecordWithFlags(e->evk0, s, evf));
  // With weak-support lists, the work list, the sweep-start snapshot and the
  // lists are built by one launch (inside the sweep's kernel time).
  if (with_weak) CP_CUDA(launch_work_and_weak(net->dn, net->level_ptr(level), S, S.snap, S.weak, s));
  // Mode 0: failed branches remove their value from the level at once
  // (later branches of the sweep start without it; the closure is the
  // same, since a wipe-out on a larger domain implies one on a smaller);
  // mode 1 keeps the plain Jacobi sweep as the reference path.
  u64* gs_root = e->sac_mode == 0 && !sweep_only ? net->level_ptr(level) : nullptr;
  if (tiled) {
    // Two-round branches resolved by the tiled kernel, the rest (the deep
    // list) by the general kernel; the sweep-start domains and the
    // weak-support lists counted against them come first.
    // Without the snapshot the tiled kernel reads the level itself and removes
    // nothing at it (a pure Jacobi sweep: the level does not change).
    SacScratch St = S;
    if (sweep_only) St.snap = nullptr;
    CP_CUDA(launch_sac_tile(net->dn, net->level_ptr(level), St, S.ok, net->slot_cap, net->d_stats, kTileBlock,
                            net->tile_grid, s));
    CP_CUDA(launch_sac_branches(net->dn, net->level_ptr(level), S.work, S.nwork, S.cursor, S.ok, net->d_stats,
                                e->block_sac, net->sac_grid, net->d_sac_scratch, net->sac_stride, s, S.deep,
                                S.ndeep, gs_root));
    launches += 1;
    e->launches += 1;
  } else {
    CP_CUDA(launch_sac_branches(net->dn, net->level_ptr(level), S.work, S.nwork, S.cursor, S.ok, net->d_stats,
                                e->block_sac, net->sac_grid, net->d_sac_scratch, net->sac_stride, s, nullptr,
                                nullptr, gs_root));
  }
  CP_CUDA(cudaEventRecordWithFlags(e->evk1, s, evf));
  // The round's stats go straight into host-mapped memory (from the commit
  // kernel's last block, or a one-block kernel), not by a copy node that
  // would queue behind other engines' transfers.
  if (!sweep_only) {
    CP_CUDA(launch_commit(net->dn, net->level_ptr(level), S, net->d_stats, net->dh_stats, 2, net->dh_dom, s));
  } else {
    CP_CUDA(launch_stats_out(net->d_stats, net->dh_stats, 2, s));
  }
  launches += 3;  // the work list (with the weak lists where there are any), the general branch kernel,
  e->launches += 3;  // and the commit or stats kernel
  return CP_OK;
}

// A round as one graph launch: captured on first use for this level and
// these knobs, replayed afterwards (the host's launch cost of a dozen
// operations becomes one). Rounds that must read a count on the host, and
// networks whose round cannot be captured, run uncaptured.
int sac_round(cp_net* net, int level, bool root, int& launches) {
  cp_engine* e = net->e;
  cudaStream_t s = e->stream;
  if (!e->sac_graphs || net->sac_graph_off || !(root || net->prefer_grid))
    return sac_round_launches(net, level, root, launches, false);
  const std::array<int64_t, 10> key = {level, e->sac_mode, e->block_sac, e->chunk, e->block_node,
                                       net->sac_grid, net->tile_grid, net->slot_cap, net->front_blocks, e->wait_ns};
  if (key != net->sac_key) {
    net->drop_sac_graphs();
    net->sac_key = key;
  }
  const int k = root ? 0 : 1;
  if (!net->sac_exec[k]) {
    cudaGraph_t graph = nullptr;
    CP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = e->launches;
    int cnt = 0;
    const int rc = sac_round_launches(net, level, root, cnt, true);
    e->launches = l0;
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    cudaError_t ie = cudaErrorUnknown;
    if (rc == CP_OK && ce == cudaSuccess && graph) ie = cudaGraphInstantiate(&net->sac_exec[k], graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      cudaGetLastError();
      net->sac_exec[k] = nullptr;
      net->sac_graph_off = true;
      return sac_round_launches(net, level, root, launches, false);
    }
    net->sac_launches[k] = cnt;
  }
  CP_CUDA(cudaGraphLaunch(net->sac_exec[k], s));
  launches += net->sac_launches[k];
  e->launches += net->sac_launches[k];
  return CP_OK;
}

// Waits for the round's stats copy and checks the device-side error flags.
int sac_round_wait(cp_net* net) {
  CP_CUDA(cudaStreamSynchronize(net->e->stream));
  for (int i = 0; i < 2; ++i) {
    if (net->h_stats[i].grid_err) return fail(CP_E_TIMEOUT, "device grid barrier wait ran out");
    if (net->h_stats[i].error) return fail(net->h_stats[i].error, "device-side check failed (round limit)");
  }
  return CP_OK;
}

}  // namespace

extern "C" {

// SAC1 in two halves: begin queues the first round (level AC + sweep) and
// returns; end waits for it and runs the further sweeps the host decides on.
static int sac1_begin(cp_net* net, int level) {
  if (!net) return fail(CP_E_ARG, "null net");
  CP_TRY(check_level(net, level));
  if (net->sac_pending_level >= 0) return fail(CP_E_STATE, "a SAC1 call on this network is still open");
  cp_engine* e = net->e;
  cudaStream_t s = e->stream;
  net->sac_pending_launches = 0;
  CP_CUDA(cudaEventRecord(e->ev0, s));
  CP_TRY(sac_round(net, level, true, net->sac_pending_launches));
  // The end of this round on the device; the last record (the round after
  // which the host stops) closes device_ms without the host's reaction time.
  CP_CUDA(cudaEventRecord(e->ev1, s));
  net->sac_pending_level = level;
  return CP_OK;
}

static int sac1_end(cp_net* net, cp_stats* st, uint64_t* domains = nullptr) {
  if (!net) return fail(CP_E_ARG, "null net");
  if (net->sac_pending_level < 0) return fail(CP_E_STATE, "no SAC1 call open on this network");
  const int level = net->sac_pending_level;
  net->sac_pending_level = -1;
  cp_engine* e = net->e;
  cudaStream_t s = e->stream;
  Acc acc;
  int launches = net->sac_pending_launches;
  bool inconsistent = false;
  int sweeps = 1;
  double kernel_ms = 0, kernel_bytes = 0;
  for (;;) {
    CP_TRY(sac_round_wait(net));
    acc.add(net->h_stats[1], 0);  // the level AC before this sweep
    if (net->h_stats[1].inconsistent) {
      inconsistent = true;
      --sweeps;  // the sweep queued behind the wipe-out does not count
      break;
    }
    const KStats k = net->h_stats[0];
    {
      // Values removed at the level are the failed tests; removals inside the
      // branches' private domain copies are not deletions of this call.
      KStats kl = k;
      kl.deletions = k.removed;
      acc.add(kl, 0);
    }
    {
      float kms = 0;
      CP_CUDA(cudaEventElapsedTime(&kms, e->evk0, e->evk1));
      kernel_ms += kms;
      Acc ka;
      KStats kk = k;
      kk.deletions -= kk.removed;  // commit-kernel removals are not the branch kernel's
      ka.add(kk, 0);
      kernel_bytes += alg_bytes(net, ka, static_cast<int64_t>(k.branches));
    }
    if (k.removed == 0) break;
    ++sweeps;
    CP_TRY(sac_round(net, level, false, launches));
    CP_CUDA(cudaEventRecord(e->ev1, s));
  }
  CP_CUDA(cudaEventSynchronize(e->ev1));
  if (domains) {
    // The last sweep removed nothing, so its commit kernel left the level in
    // h_dom; otherwise (a wipe-out) the level is read back.
    if (!inconsistent && net->h_stats[0].removed == 0) {
      for (int x = 0; x < net->n; ++x)
        for (int w = 0; w < net->W_user; ++w)
          domains[static_cast<size_t>(x) * net->W_user + w] = net->h_dom[static_cast<size_t>(x) * net->W + w];
    } else {
      CP_TRY(fetch_level(net, level, domains));
    }
  }
  if (st) {
    acc.s.inconsistent = inconsistent ? 1 : 0;
    acc.s.deletions = acc.dels;
    acc.s.sweeps = sweeps;
    acc.s.launches = launches;
    acc.s.device_ms = elapsed_ms(e);
    acc.s.alg_bytes = alg_bytes(net, acc, acc.s.branches);
    acc.s.kernel_ms = kernel_ms;
    acc.s.kernel_bytes = kernel_bytes;
    *st = acc.s;
  }
  return CP_OK;
}

int cp_enforce_sac1(cp_net* net, int level, cp_stats* st) {
  CP_TRY(sac1_begin(net, level));
  return sac1_end(net, st);
}

int cp_enforce_sac1_begin(cp_net* net, int level) { return sac1_begin(net, level); }

int cp_enforce_sac1_end(cp_net* net, cp_stats* st) { return sac1_end(net, st); }

int cp_enforce_sac1_end_domains(cp_net* net, cp_stats* st, uint64_t* domains) {
  if (!domains) return fail(CP_E_ARG, "null domains");
  return sac1_end(net, st, domains);
}

int cp_sac_sweep(cp_net* net, int level, uint64_t* verdict, int64_t* deep, cp_stats* st) {
  if (!net || !verdict) return fail(CP_E_ARG, "null argument");
  CP_TRY(check_level(net, level));
  cp_engine* e = net->e;
  cudaStream_t s = e->stream;
  int launches = 0;
  CP_CUDA(cudaEventRecord(e->ev0, s));
  CP_TRY(sac_round_launches(net, level, true, launches, false, true));
  CP_CUDA(cudaEventRecord(e->ev1, s));
  CP_TRY(sac_round_wait(net));
  const KStats lac = net->h_stats[1], k = net->h_stats[0];
  const int W = net->W_user, Wi = net->W;
  std::fill(verdict, verdict + static_cast<size_t>(net->n) * W, 0ull);
  int cnt[2] = {0, 0};  // nwork, ndeep
  if (!lac.inconsistent) {
    CP_CUDA(cudaMemcpyAsync(&cnt[0], net->S.nwork, sizeof(int), cudaMemcpyDeviceToHost, s));
    CP_CUDA(cudaMemcpyAsync(&cnt[1], net->S.ndeep, sizeof(int), cudaMemcpyDeviceToHost, s));
    CP_CUDA(cudaStreamSynchronize(s));
    std::vector<int2> work(cnt[0]);
    std::vector<uint8_t> ok(cnt[0]);
    if (cnt[0]) {
      CP_CUDA(cudaMemcpyAsync(work.data(), net->S.work, cnt[0] * sizeof(int2), cudaMemcpyDeviceToHost, s));
      CP_CUDA(cudaMemcpyAsync(ok.data(), net->S.ok, cnt[0], cudaMemcpyDeviceToHost, s));
      CP_CUDA(cudaStreamSynchronize(s));
    }
    for (int i = 0; i < cnt[0]; ++i) {
      if (!ok[i]) continue;
      const int x = work[i].x, a = work[i].y;
      if ((a >> 6) < W) verdict[static_cast<size_t>(x) * W + (a >> 6)] |= 1ull << (a & 63);
    }
  }
  (void)Wi;
  if (deep) *deep = (e->sac_mode == 0 && net->tile_grid > 0) ? cnt[1] : 0;
  if (st) {
    Acc a;
    a.add(lac, 0);
    a.add(k, 0);
    a.s.inconsistent = lac.inconsistent;
    a.s.deletions = static_cast<int64_t>(lac.deletions);
    a.s.sweeps = lac.inconsistent ? 0 : 1;
    a.s.launches = launches;
    a.s.device_ms = elapsed_ms(e);
    a.s.alg_bytes = alg_bytes(net, a, a.s.branches);
    float kms = 0;
    CP_CUDA(cudaEventElapsedTime(&kms, e->evk0, e->evk1));
    a.s.kernel_ms = kms;
    Acc ka;
    ka.add(k, 0);
    a.s.kernel_bytes = alg_bytes(net, ka, static_cast<int64_t>(k.branches));
    *st = a.s;
  }
  return CP_OK;
}

int cp_sac_tiles(cp_net* net, int level, int ntiles, const int* tile_x, const int* tile_c1, const int* tile_c2,
                 int mode, uint64_t* out, double* ms) {
  if (!net || ntiles < 0 || (ntiles > 0 && (!tile_x || !tile_c1 || !tile_c2 || !out)))
    return fail(CP_E_ARG, "null argument");
  CP_TRY(check_level(net, level));
  if (mode != 0 && mode != 1) return fail(CP_E_ARG, "mode must be 0 (bitwise) or 1 (tensor cores)");
  if (net->W > 2 || net->dn.nt != 0) return fail(CP_E_UNSUPPORTED, "tiles need a binary network of at most 128 values");
  const int nb = static_cast<int>(net->bx.size());
  std::vector<SacTile> tiles(ntiles);
  for (int t = 0; t < ntiles; ++t) {
    const int x = tile_x[t], c1 = tile_c1[t], c2 = tile_c2[t];
    if (c1 < 0 || c1 >= nb || c2 < 0 || c2 >= nb) return fail(CP_E_ARG, "constraint out of range");
    const bool x_first = net->bx[c1] == x;
    if (!x_first && net->by[c1] != x) return fail(CP_E_ARG, "constraint c1 does not contain x");
    const int y = x_first ? net->by[c1] : net->bx[c1];
    const bool y_first = net->bx[c2] == y;
    if (!y_first && net->by[c2] != y) return fail(CP_E_ARG, "constraint c2 does not contain y");
    const int z = y_first ? net->by[c2] : net->bx[c2];
    SacTile& T = tiles[t];
    // Rows of x over y: the A block when x is the first variable of c1, else
    // the B block; likewise rows of z over y in c2.
    T.xy = static_cast<u32>(x_first ? net->offA[c1] : net->offB[c1]);
    T.zy = static_cast<u32>(y_first ? net->offB[c2] : net->offA[c2]);
    T.y = y;
    T.z = z;
    T.dx = net->dom[x];
    T.dz = net->dom[z];
    T.pad0 = T.pad1 = 0;
  }
  if (ntiles == 0) {
    if (ms) *ms = 0.0;
    return CP_OK;
  }
  cp_engine* e = net->e;
  cudaStream_t s = e->stream;
  const size_t out_words = static_cast<size_t>(ntiles) * 128 * 2;
  void *d_tiles = nullptr, *d_out = nullptr, *d_err = nullptr;
  int rc = e->dev_alloc(&d_tiles, tiles.size() * sizeof(SacTile));
  if (rc == CP_OK) rc = e->dev_alloc(&d_out, out_words * 8);
  if (rc == CP_OK) rc = e->dev_alloc(&d_err, sizeof(int));
  int h_err = 0;
  float kms = 0;
  if (rc == CP_OK) {
    cudaError_t ce = cudaMemcpyAsync(d_tiles, tiles.data(), tiles.size() * sizeof(SacTile), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(d_err, 0, sizeof(int), s);
    if (ce == cudaSuccess) ce = cudaEventRecord(e->evk0, s);
    if (ce == cudaSuccess)
      ce = mode == 0 ? launch_tiles_bitwise(net->W, net->d_rel, net->level_ptr(level),
                                            static_cast<const SacTile*>(d_tiles), ntiles, static_cast<u64*>(d_out),
                                            e->sm_count, s)
                     : launch_tiles_tc(net->W, net->d_rel, net->level_ptr(level), static_cast<const SacTile*>(d_tiles),
                                       ntiles, static_cast<u64*>(d_out), static_cast<int*>(d_err), e->sm_count, s);
    if (ce == cudaSuccess) ce = cudaEventRecord(e->evk1, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(out, d_out, out_words * 8, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&kms, e->evk0, e->evk1);
    if (ce != cudaSuccess) rc = fail(CP_E_CUDA, std::string("cp_sac_tiles: ") + cudaGetErrorString(ce));
  }
  ++e->launches;
  for (void* p : {d_tiles, d_out, d_err})
    if (p) e->dev_free(p);
  if (rc != CP_OK) return rc;
  if (h_err) return fail(CP_E_TIMEOUT, "tensor-core product did not complete within the bounded wait");
  if (ms) *ms = kms;
  return CP_OK;
}

int cp_singletons(cp_net* net, int level, int count, const int* vars, const int* vals, uint8_t* ok, int mode,
                  cp_stats* st) {
  if (!net || (count > 0 && (!vars || !vals || !ok))) return fail(CP_E_ARG, "null argument");
  CP_TRY(check_level(net, level));
  if (count < 0 || count > net->dn.total_values) return fail(CP_E_ARG, "count out of range");
  for (int i = 0; i < count; ++i) CP_TRY(check_var_val(net, vars[i], vals[i]));
  cp_engine* e = net->e;
  cudaStream_t s = e->stream;
  std::vector<int2> pairs(count);
  for (int i = 0; i < count; ++i) pairs[i] = make_int2(vars[i], vals[i]);
  if (count) CP_CUDA(cudaMemcpyAsync(net->S.work, pairs.data(), count * sizeof(int2), cudaMemcpyHostToDevice, s));
  net->h_sizes[0] = count;
  CP_CUDA(cudaMemcpyAsync(net->S.nwork, net->h_sizes, sizeof(int), cudaMemcpyHostToDevice, s));
  CP_CUDA(cudaMemsetAsync(net->S.cursor, 0, sizeof(int), s));
  CP_CUDA(cudaStreamSynchronize(s));
  CP_TRY(stats_begin(net));
  int launches = 0;
  CP_CUDA(cudaEventRecord(e->ev0, s));
  uint8_t* d_ok = nullptr;
  if (mode == 0) {
    CP_CUDA(launch_sac_branches(net->dn, net->level_ptr(level), net->S.work, net->S.nwork, net->S.cursor, net->S.ok,
                                net->d_stats, e->block_sac, net->sac_grid, net->d_sac_scratch, net->sac_stride, s));
    ++launches;
    d_ok = net->S.ok;
  } else if (mode == 1) {
    for (int i = 0; i < count; ++i) {
      CP_CUDA(launch_node(net->dn, net->d_levels, level, level, kOpSingleton, vars[i], vals[i], nullptr, 0,
                          net->d_stats, net->d_ok1 + i, e->block_node,
                          net->cta_in_smem ? nullptr : net->d_cta_scratch, s));
      ++launches;
    }
    d_ok = net->d_ok1;
  } else {
    return fail(CP_E_ARG, "mode must be 0 (batched) or 1 (one launch per test)");
  }
  e->launches += launches;
  CP_CUDA(cudaEventRecord(e->ev1, s));
  if (count) CP_CUDA(cudaMemcpyAsync(ok, d_ok, count, cudaMemcpyDeviceToHost, s));
  CP_TRY(stats_fetch(net));
  if (st) {
    Acc a;
    a.add(*net->h_stats, launches);
    if (mode == 1) {
      a.s.branches = count;
      a.s.fixpoints = count;
    }
    a.s.deletions = 0;
    a.s.device_ms = elapsed_ms(e);
    a.s.alg_bytes = alg_bytes(net, a, a.s.branches);
    a.s.kernel_ms = a.s.device_ms;
    a.s.kernel_bytes = a.s.alg_bytes;
    *st = a.s;
  }
  return CP_OK;
}

}  // extern "C"

// ===========================================================================
// Search
// ===========================================================================
namespace {

// Device-resident node operations for the search loops: each returns the
// consistency verdict and leaves the resulting level mirrored in h_dom.
struct NodeRunner {
  cp_net* net;
  int64_t propagations = 0;

  int node(int op, int src, int dst, int var, int val, bool& consistent) {
    cp_engine* e = net->e;
    cudaStream_t s = e->stream;
    CP_TRY(stats_begin(net));
    if (!net->prefer_grid) {
      CP_CUDA(launch_node(net->dn, net->d_levels, src, dst, op, var, val, nullptr, 0, net->d_stats, nullptr,
                          e->block_node, net->cta_in_smem ? nullptr : net->d_cta_scratch, s));
      ++e->launches;
    } else {
      int launches = 0;
      if (op == kOpRoot) {
        CP_TRY(run_ac(net, src, nullptr, 0, launches));
      } else {
        if (src != dst)
          CP_CUDA(cudaMemcpyAsync(net->level_ptr(dst), net->level_ptr(src), static_cast<size_t>(net->n) * net->W * 8,
                                  cudaMemcpyDeviceToDevice, s));
        CP_CUDA(launch_level_edit(net->dn, net->level_ptr(dst), var, val, op == kOpRefute ? kOpRefute : kOpAssign, s));
        ++e->launches;
        net->h_sizes[0] = var;
        CP_CUDA(cudaMemcpyAsync(net->d_evt, net->h_sizes, sizeof(int), cudaMemcpyHostToDevice, s));
        CP_TRY(run_ac(net, dst, net->d_evt, 1, launches));
      }
    }
    ++propagations;
    CP_CUDA(cudaMemcpyAsync(net->h_dom, net->level_ptr(dst), static_cast<size_t>(net->n) * net->W * 8,
                            cudaMemcpyDeviceToHost, s));
    CP_TRY(stats_fetch(net));
    consistent = net->h_stats->inconsistent == 0;
    return CP_OK;
  }
  int size(int x) const {
    int sz = 0;
    for (int w = 0; w < net->W; ++w) sz += __builtin_popcountll(net->h_dom[static_cast<size_t>(x) * net->W + w]);
    return sz;
  }
  int head(int x) const {
    for (int w = 0; w < net->W; ++w) {
      const u64 v = net->h_dom[static_cast<size_t>(x) * net->W + w];
      if (v) return w * 64 + __builtin_ctzll(v);
    }
    return -1;
  }
  int next(int x, int a) const {
    for (int b = a + 1; b < net->dom[x]; ++b)
      if ((net->h_dom[static_cast<size_t>(x) * net->W + (b >> 6)] >> (b & 63)) & 1ull) return b;
    return -1;
  }
};

// MAC::enforce (src/MAC.cpp:100-165) with the per-level "assigned" flags of
// IntVar (include/Network.h:183, src/Network.cpp:112-118, 235-256) and
// AssignedStack (src/Solver.cpp:36-56, 114-116), which decide the variable
// order; only domains live on the device.
class DeviceMAC {
 public:
  DeviceMAC(cp_net* net, int varh, int valh) : R{net}, n_(net->n), L_(net->levels), varh_(varh), valh_(valh) {
    assigned_.assign(static_cast<size_t>(L_) * n_, 0);
    top_.assign(n_, 0);
    if (varh_ == 6) {
      weight_.assign(net->bx.size(), 1.0);  // Tabular::weight starts at 1 (src/Network.cpp:303)
      cons_of_.resize(n_);
      for (size_t c = 0; c < net->bx.size(); ++c) {
        cons_of_[net->bx[c]].push_back(static_cast<int>(c));
        cons_of_[net->by[c]].push_back(static_cast<int>(c));
      }
    }
  }

  int solve(int64_t time_limit_ms, cp_search_result* res, int* solution) {
    const auto t0 = std::chrono::steady_clock::now();
    auto elapsed = [&]() {
      return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    };
    *res = cp_search_result{};
    bool consistent = false;
    CP_TRY(node(kOpRoot, 0, 0, 0, 0, consistent));
    if (!consistent) return finish(res, 0, elapsed());
    for (;;) {
      if (elapsed() > double(time_limit_ms)) return finish(res, 2, elapsed());
      const int p = static_cast<int>(I_.size());
      if (p + 1 >= L_) return fail(CP_E_ARG, "level stack too shallow for the search");
      const int var = select_var(p);
      if (var < 0) return fail(CP_E_STATE, "no variable to branch on");
      const int val = R.head(var);
      new_level(p);
      push(var, val);
      ++res->num_positive;
      const int lv = static_cast<int>(I_.size());
      A(lv)[var] = 1;  // IntVar::ReduceTo marks the variable assigned
      CP_TRY(node(kOpAssign, p, lv, var, val, consistent));
      if (consistent && lv == n_) {
        for (int x = 0; x < n_; ++x) solution[x] = R.head(x);
        return finish(res, 1, elapsed());
      }
      while (!consistent && !I_.empty()) {
        const auto va = pop();
        const int q = static_cast<int>(I_.size());
        back_to(q);
        ++res->num_negative;
        CP_TRY(node(kOpRefute, q, q, va.first, va.second, consistent));
        update_model_assigned();
      }
      if (!consistent) return finish(res, 0, elapsed());
    }
  }

 private:
  NodeRunner R;
  int n_, L_, varh_, valh_;
  std::vector<char> assigned_;
  std::vector<int> top_;
  std::vector<std::pair<int, int>> I_;
  std::vector<double> weight_;           // dom/wdeg constraint weights
  std::vector<std::vector<int>> cons_of_;  // dom/wdeg: constraints of each variable

  char* A(int p) { return &assigned_[static_cast<size_t>(p) * n_]; }

  // One node (the AC call of MAC::enforce); under dom/wdeg a failing node's
  // propagation is replayed in the reference's sequential order on the
  // node's starting domains (copied before the node runs) to find the
  // constraint whose weight rises.
  int node(int op, int src, int dst, int var, int val, bool& consistent) {
    cp_net* net = R.net;
    cudaStream_t s = net->e->stream;
    const size_t words = static_cast<size_t>(n_) * net->W;
    if (varh_ == 6) {
      CP_TRY(replay_scratch());
      CP_CUDA(cudaMemcpyAsync(net->d_replay_dom, net->level_ptr(src), words * 8, cudaMemcpyDeviceToDevice, s));
    }
    CP_TRY(R.node(op, src, dst, var, val, consistent));
    if (varh_ == 6 && !consistent) {
      // The flags the AC call sees: the level it runs at.
      const int lv = op == kOpAssign ? dst : src;
      std::memcpy(net->h_sizes, A(lv), static_cast<size_t>(n_));
      CP_CUDA(cudaMemcpyAsync(net->d_replay_assigned, net->h_sizes, static_cast<size_t>(n_), cudaMemcpyHostToDevice, s));
      CP_CUDA(launch_ac3_replay(net->dn, net->d_arc_con, net->d_bx, net->d_by, net->d_replay_dom,
                                net->d_replay_assigned, op, var, val, net->replay, net->d_replay_out, s));
      ++net->e->launches;
      int c = -1;
      CP_CUDA(cudaMemcpyAsync(&net->h_sizes[0], net->d_replay_out, sizeof(int), cudaMemcpyDeviceToHost, s));
      CP_CUDA(cudaStreamSynchronize(s));
      c = net->h_sizes[0];
      if (c >= 0 && c < static_cast<int>(weight_.size())) weight_[c] += 1.0;
    }
    return CP_OK;
  }
  int replay_scratch() {
    cp_net* net = R.net;
    if (net->d_replay_out) return CP_OK;
    const size_t nb = std::max<size_t>(1, net->bx.size());
    CP_TRY(net->alloc(&net->replay.stamp_var, static_cast<size_t>(n_)));
    CP_TRY(net->alloc(&net->replay.stamp_tab, nb));
    CP_TRY(net->alloc(&net->replay.q, static_cast<size_t>(n_) + 1));
    CP_TRY(net->alloc(&net->replay.inq, static_cast<size_t>(n_)));
    CP_TRY(net->alloc(&net->d_replay_dom, static_cast<size_t>(n_) * net->W));
    CP_TRY(net->alloc(&net->d_replay_assigned, static_cast<size_t>(n_)));
    CP_TRY(net->alloc(&net->d_replay_out, 1));
    return CP_OK;
  }
  int finish(cp_search_result* res, int status, double ms) {
    res->status = status;
    res->propagations = R.propagations;
    res->solve_ms = ms;
    return CP_OK;
  }
  // VRH_DOM_MIN (src/MAC.cpp:357-365): first unassigned variable of strictly
  // smaller size; VRH_LEX (:366-368); VRH_DOM_DEG_MIN (:371-386): the same
  // with the integer key size / |neighbourhood| (-1 without neighbours).
  // VRH_DOM_WDEG_MIN (:387-408): |D(v)| over the summed weights of v's
  // constraints that have another unassigned variable, -1 when |D(v)| = 1 or
  // the sum is 0; the first strict minimum, in doubles as the reference.
  int select_var(int p) {
    if (varh_ == 0) return static_cast<int>(I_.size()) + 1 < n_ ? static_cast<int>(I_.size()) + 1 : -1;
    int var = -1;
    double min_size = 1e300;
    for (int v = 0; v < n_; ++v) {
      if (A(p)[v]) continue;
      double key;
      if (varh_ == 6) {
        double w = 0.0;
        for (int c : cons_of_[v]) {
          const int free = (A(p)[R.net->bx[c]] ? 0 : 1) + (A(p)[R.net->by[c]] ? 0 : 1);
          if (free > 1) w += weight_[c];
        }
        const int sz = R.size(v);
        key = (sz == 1 || w == 0.0) ? -1.0 : sz / w;
      } else {
        const int deg = R.net->nbr_count[v];
        key = varh_ == 4 ? (deg == 0 ? -1 : R.size(v) / deg) : R.size(v);
      }
      if (key < min_size) {
        min_size = key;
        var = v;
      }
    }
    return var;
  }
  void new_level(int src) {
    std::copy(A(src), A(src) + n_, A(src + 1));
    std::fill(top_.begin(), top_.end(), src);
  }
  void back_to(int dest) {
    for (int v = 0; v < n_; ++v) {
      for (int i = dest; i <= top_[v]; ++i) A(i)[v] = 0;
      top_[v] = dest;
    }
  }
  void push(int v, int a) {
    I_.emplace_back(v, a);
    A(static_cast<int>(I_.size()))[v] = 1;
  }
  std::pair<int, int> pop() {
    const auto va = I_.back();
    I_.pop_back();
    A(static_cast<int>(I_.size()))[va.first] = 0;
    return va;
  }
  void update_model_assigned() {
    for (const auto& va : I_) A(static_cast<int>(I_.size()))[va.first] = 1;
  }
};

// GModelSolver::Solve / Search (src/GModelSolver.cu:31-189): d-way search,
// smallest domain among variables with more than one value
// (GModel::GetMinDomainVar, src/GModel.cu:1553-1572), values in increasing
// order, one GAC per node.
class DeviceGSolver {
 public:
  explicit DeviceGSolver(cp_net* net) : R{net}, n_(net->n) {}
  int solve(int64_t time_limit_ms, cp_search_result* res, int* solution) {
    t0_ = std::chrono::steady_clock::now();
    limit_ = time_limit_ms;
    *res = cp_search_result{};
    res_ = res;
    sol_ = solution;
    bool consistent = false;
    CP_TRY(R.node(kOpRoot, 0, 0, 0, 0, consistent));
    if (!consistent) return finish(0);
    if (fully_assigned()) {
      extract();
      return finish(1);
    }
    bool stop = false;
    CP_TRY(search(0, stop));
    return finish(found_ ? 1 : (timed_out_ ? 2 : 0));
  }

 private:
  NodeRunner R;
  int n_;
  std::chrono::steady_clock::time_point t0_;
  int64_t limit_ = 0;
  cp_search_result* res_ = nullptr;
  int* sol_ = nullptr;
  bool found_ = false, timed_out_ = false;

  double elapsed() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0_).count();
  }
  int finish(int status) {
    res_->status = status;
    res_->propagations = R.propagations;
    res_->solve_ms = elapsed();
    return CP_OK;
  }
  bool fully_assigned() const {
    for (int x = 0; x < n_; ++x)
      if (R.size(x) != 1) return false;
    return true;
  }
  void extract() {
    for (int x = 0; x < n_; ++x) sol_[x] = R.head(x);
    found_ = true;
  }
  int search(int level, bool& stop) {
    if (limit_ > 0 && elapsed() >= double(limit_)) {
      timed_out_ = true;
      stop = true;
      return CP_OK;
    }
    if (level + 1 >= R.net->levels) return fail(CP_E_ARG, "level stack too shallow for the search");
    // R.h_dom mirrors `level` here.
    std::vector<u64> here(R.net->h_dom, R.net->h_dom + static_cast<size_t>(n_) * R.net->W);
    int var = -1, min_size = 1 << 30;
    for (int x = 0; x < n_; ++x) {
      const int sz = R.size(x);
      if (sz > 1 && sz < min_size) {
        min_size = sz;
        var = x;
      }
    }
    if (var < 0) {
      if (fully_assigned()) {
        extract();
        stop = true;
      }
      return CP_OK;
    }
    for (int val = R.head(var); val != -1;) {
      ++res_->num_positive;
      bool consistent = false;
      CP_TRY(R.node(kOpAssign, level, level + 1, var, val, consistent));
      if (!consistent) {
        ++res_->num_negative;
      } else {
        CP_TRY(search(level + 1, stop));
        if (stop) return CP_OK;
      }
      std::copy(here.begin(), here.end(), R.net->h_dom);
      val = R.next(var, val);
    }
    return CP_OK;
  }
};

}  // namespace

// ---- device-resident MAC searches --------------------------------------
// A launch runs each search for at most this long; searches still open are
// resumed by the next launch, so no kernel of the search runs for long.
constexpr long long kMacSliceNs = 50ll * 1000 * 1000;

struct MacSpec {
  cp_net* net = nullptr;
  const u64* init = nullptr;  // domains before the choices
  u64* stack = nullptr;       // level stack (null: allocated for the search)
  int levels = 0;
  std::vector<int2> choices;
};

struct cp_mac_batch {
  cp_engine* e = nullptr;
  int k = 0;
  std::vector<int> n_of;
  std::vector<int64_t> sol_off;
  std::vector<void*> allocs;  // device pool blocks
  void* h_block = nullptr;    // host-mapped: MacOut[k], then the solutions
  size_t h_bytes = 0;
  void* stage = nullptr;      // pinned staging of the job descriptors
  size_t stage_bytes = 0;
  MacOut* outs = nullptr;
  int* sols = nullptr;
  std::vector<uint8_t> reported;
  std::vector<cp_search_result> res;
  cudaEvent_t ev = nullptr;
  std::chrono::steady_clock::time_point t0;
  // Launch parameters, kept for the relaunches that resume suspended searches.
  DevNet* d_dn = nullptr;
  MacJob* d_jobs = nullptr;
  int* d_cursor = nullptr;
  MacOut* d_outs = nullptr;
  int block = 0, grid = 0;
  size_t smem = 0, gstride = 0;
  char* gscratch = nullptr;
  int launches = 0;
  int launch() {
    cudaStream_t s = e->stream;
    CP_CUDA(cudaMemsetAsync(d_cursor, 0, sizeof(int), s));
    CP_CUDA(launch_mac(d_dn, d_jobs, k, d_cursor, d_outs, block, grid, smem, gscratch, gstride, kMacSliceNs, s));
    ++e->launches;
    ++launches;
    CP_CUDA(cudaEventRecord(ev, s));
    return CP_OK;
  }
  ~cp_mac_batch() {
    if (!e) return;
    if (ev) {
      cudaEventSynchronize(ev);
      cudaEventDestroy(ev);
    }
    for (void* p : allocs) e->dev_free(p);
    e->mapped_put(h_block, h_bytes);
    e->pinned_put(stage, stage_bytes);
    --e->live_nets;
    if (e->closed && e->live_nets == 0) engine_free(e);
  }
};

namespace {

// Lays out and launches one k_mac grid over the specs.
int mac_start(cp_engine* e, std::vector<MacSpec>& specs, int varh, int64_t time_limit_ms, cp_mac_batch* b) {
  CP_CUDA(cudaSetDevice(e->device));
  cudaStream_t s = e->stream;
  const int k = static_cast<int>(specs.size());
  b->e = e;
  ++e->live_nets;  // a MAC batch holds the engine like a network does
  b->k = k;
  b->n_of.resize(k);
  b->sol_off.resize(k + 1, 0);
  b->reported.assign(k, 0);
  b->res.resize(k);
  size_t max_state = 0;
  for (int i = 0; i < k; ++i) {
    b->n_of[i] = specs[i].net->n;
    b->sol_off[i + 1] = b->sol_off[i] + specs[i].net->n;
    max_state = std::max(max_state, cta_state_bytes(specs[i].net->dn));
  }
  // Host-visible results.
  const size_t out_bytes = (sizeof(MacOut) * static_cast<size_t>(k) + 255) & ~size_t(255);
  b->h_bytes = out_bytes + static_cast<size_t>(b->sol_off[k]) * sizeof(int);
  CP_TRY(e->mapped_get(b->h_bytes, &b->h_block));
  std::memset(b->h_block, 0, b->h_bytes);
  void* d_host = nullptr;
  CP_CUDA(cudaHostGetDevicePointer(&d_host, b->h_block, 0));
  b->outs = static_cast<MacOut*>(b->h_block);
  b->sols = reinterpret_cast<int*>(static_cast<char*>(b->h_block) + out_bytes);
  MacOut* d_outs = static_cast<MacOut*>(d_host);
  int* d_sols = reinterpret_cast<int*>(static_cast<char*>(d_host) + out_bytes);
  // Device block: [networks | jobs | choices | cursor] copied, then scratch.
  std::vector<DevNet> dn(k);
  std::vector<MacJob> jobs(k);
  std::vector<int2> ch;
  std::vector<int64_t> ch_off(k + 1, 0);
  // Small work items when the searches leave SMs idle (unless a chunk was
  // set with cp_engine_set_tuning): a node's fixpoint then spreads the arcs
  // of a changed variable over the CTA's warps instead of walking chunk of
  // them in one warp. One arc per item on networks of up to 1024 arcs (one
  // 500-arc cfg1 search on one GB300: 0.41 ms vs 0.45 ms at four arcs and
  // 0.65 ms at eight), one grouped pass (four arcs of one-word domains, two
  // of two-word ones) on larger ones (46 k vs 42 k nodes/s at 1600 arcs,
  // 18.3 k vs 16.2 k at 4000).
  const bool spread = k < e->sm_count && e->chunk == 0;
  for (int i = 0; i < k; ++i) {
    dn[i] = specs[i].net->dn;
    if (spread) dn[i].chunk = 2 * dn[i].nb <= 1024 ? 1 : 32 / arc_group_lanes(dn[i].W);
    ch.insert(ch.end(), specs[i].choices.begin(), specs[i].choices.end());
    ch_off[i + 1] = static_cast<int64_t>(ch.size());
  }
  int zero = 0;
  DevNet* d_dn = nullptr;
  MacJob* d_jobs = nullptr;
  int2* d_ch = nullptr;
  int* d_cursor = nullptr;
  MetaPack mp;
  mp.add(&d_dn, dn.data(), k);
  mp.add(&d_jobs, jobs.data(), k);  // filled below, before the copy
  mp.add(&d_ch, ch.data(), ch.size());
  mp.add(&d_cursor, &zero, 1);
  size_t scratch = 0;
  std::vector<size_t> off_stack(k), off_assigned(k), off_path(k);
  auto up = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t off_state = scratch;
  scratch += up(sizeof(MacState) * static_cast<size_t>(k));
  for (int i = 0; i < k; ++i) {
    const cp_net* n = specs[i].net;
    const size_t words = static_cast<size_t>(n->n) * n->W;
    off_stack[i] = scratch;
    if (!specs[i].stack) scratch += up(static_cast<size_t>(specs[i].levels) * words * 8);
    off_assigned[i] = scratch;
    scratch += up(static_cast<size_t>(specs[i].levels) * n->n);
    off_path[i] = scratch;
    scratch += up(static_cast<size_t>(n->n + 1) * sizeof(int2));
  }
  // CTA state: shared memory when the largest fits, else per-CTA scratch.
  const bool smem_mode = max_state + 2048 <= e->smem_optin;
  // CTA size (measured on one GB300): many searches of small networks run
  // best as many small CTAs (64 threads: 163 k cfg1 searches/s vs 120 k at
  // 512); a few searches, or large networks, as wide CTAs (512 threads:
  // 1.65x the node rate of 256 on networks of a few thousand arcs).
  int max_inc = 0;
  for (const MacSpec& sp : specs) max_inc = std::max(max_inc, 2 * sp.net->nb + sp.net->nt);
  const int block = e->search_block > 0 ? e->search_block : (max_inc <= 2048 && k >= 2 * e->sm_count) ? 64 : 512;
  const int per_sm = mac_blocks_per_sm(block, smem_mode ? max_state : 0);
  if (per_sm < 1) return fail(CP_E_UNSUPPORTED, "MAC kernel does not fit on an SM");
  const int grid = std::min(k, per_sm * e->sm_count);
  const size_t gstride = smem_mode ? 0 : up(max_state);
  const size_t g_off = scratch;
  scratch += gstride * static_cast<size_t>(grid);
  char* d_block = nullptr;
  {
    void* raw = nullptr;
    CP_TRY(e->dev_alloc(&raw, mp.total + scratch + 256));
    b->allocs.push_back(raw);
    d_block = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(raw) + 255) & ~uintptr_t(255));
  }
  char* d_scratch = d_block + mp.total;
  const long long limit_ns = time_limit_ms > 0 ? static_cast<long long>(time_limit_ms) * 1000000ll : 0;
  for (int i = 0; i < k; ++i) {
    MacJob& J = jobs[i];
    J.state = reinterpret_cast<MacState*>(d_scratch + off_state) + i;
    J.net = i;
    J.levels = specs[i].levels;
    J.varh = varh;
    J.nbr = specs[i].net->d_nbr;
    J.n_choice = static_cast<int>(ch_off[i + 1] - ch_off[i]);
    J.init = specs[i].init;
    J.stack_dom = specs[i].stack ? specs[i].stack : reinterpret_cast<u64*>(d_scratch + off_stack[i]);
    J.assigned = reinterpret_cast<uint8_t*>(d_scratch + off_assigned[i]);
    J.path = reinterpret_cast<int2*>(d_scratch + off_path[i]);
    J.choices = nullptr;  // set from the packed block below
    J.solution = d_sols + b->sol_off[i];
    J.limit_ns = limit_ns;
  }
  // The staging block stays with the batch until the copy has surely ended.
  b->stage_bytes = mp.total;
  CP_TRY(e->pinned_get(mp.total, &b->stage));
  for (const auto& q : mp.parts) *q.dst = d_block + q.off;
  for (int i = 0; i < k; ++i) jobs[i].choices = jobs[i].n_choice ? d_ch + ch_off[i] : nullptr;
  for (const auto& q : mp.parts)
    if (q.bytes) std::memcpy(static_cast<char*>(b->stage) + q.off, q.src, q.bytes);
  CP_CUDA(cudaMemcpyAsync(d_block, b->stage, mp.total, cudaMemcpyHostToDevice, s));
  CP_CUDA(cudaMemsetAsync(d_scratch + off_state, 0, sizeof(MacState) * static_cast<size_t>(k), s));
  CP_CUDA(cudaEventCreateWithFlags(&b->ev, cudaEventDisableTiming));
  b->t0 = std::chrono::steady_clock::now();
  b->d_dn = d_dn;
  b->d_jobs = d_jobs;
  b->d_cursor = d_cursor;
  b->d_outs = d_outs;
  b->block = block;
  b->grid = grid;
  b->smem = smem_mode ? max_state : 0;
  b->gscratch = smem_mode ? nullptr : d_scratch + g_off;
  b->gstride = gstride;
  return b->launch();
}

}  // namespace

extern "C" {

int cp_mac_solve(cp_net* net, int var_heuristic, int val_heuristic, int64_t time_limit_ms, cp_search_result* res,
                 int* solution) {
  if (!net || !res || !solution) return fail(CP_E_ARG, "null argument");
  if (var_heuristic != 0 && var_heuristic != 1 && var_heuristic != 4 && var_heuristic != 6)
    return fail(CP_E_UNSUPPORTED,
                "variable heuristic: 0 (VRH_LEX), 1 (VRH_DOM_MIN), 4 (VRH_DOM_DEG_MIN) or 6 (VRH_DOM_WDEG_MIN)");
  if (val_heuristic != 0) return fail(CP_E_UNSUPPORTED, "value heuristic: 0 (VLH_MIN)");
  if (var_heuristic == 6 && net->dn.nt != 0)
    return fail(CP_E_UNSUPPORTED, "VRH_DOM_WDEG_MIN follows the binary AC3bit order: binary networks only");
  // dom/wdeg runs host-driven: its weights come from replays of failing nodes.
  if (net->e->search_mode == 0 && !net->prefer_grid && var_heuristic != 6) {
    // The whole search in one CTA, on the network's own level stack.
    std::vector<MacSpec> spec(1);
    spec[0].net = net;
    spec[0].init = net->level_ptr(0);
    spec[0].stack = net->d_levels;
    spec[0].levels = net->levels;
    cp_mac_batch b;
    CP_TRY(mac_start(net->e, spec, var_heuristic, time_limit_ms, &b));
    CP_TRY(cp_mac_batch_wait(&b, res));
    return cp_mac_batch_solution(&b, 0, solution);
  }
  DeviceMAC mac(net, var_heuristic, val_heuristic);
  return mac.solve(time_limit_ms, res, solution);
}

int cp_engine_set_search_mode(cp_engine* e, int mode) {
  if (!e) return fail(CP_E_ARG, "null engine");
  if (mode != 0 && mode != 1) return fail(CP_E_ARG, "search mode must be 0 (device) or 1 (host-driven)");
  e->search_mode = mode;
  return CP_OK;
}

int cp_engine_set_search_block(cp_engine* e, int block) {
  if (!e) return fail(CP_E_ARG, "null engine");
  if (block < 0 || block > 512 || block % 32) return fail(CP_E_ARG, "search block must be 0 or a multiple of 32 up to 512");
  e->search_block = block;
  return CP_OK;
}

int cp_mac_batch_start(cp_engine* e, int k, cp_net* const* nets, const int* n_choice, const int* choice_var,
                       const int* choice_val, int var_heuristic, int val_heuristic, int64_t time_limit_ms,
                       cp_mac_batch** out) {
  if (!e || !out || k < 1 || !nets) return fail(CP_E_ARG, "bad MAC batch arguments");
  if (var_heuristic != 0 && var_heuristic != 1 && var_heuristic != 4)
    return fail(CP_E_UNSUPPORTED, "variable heuristic: 0 (VRH_LEX), 1 (VRH_DOM_MIN) or 4 (VRH_DOM_DEG_MIN)");
  if (val_heuristic != 0) return fail(CP_E_UNSUPPORTED, "value heuristic: 0 (VLH_MIN)");
  std::vector<MacSpec> spec(static_cast<size_t>(k));
  int64_t c = 0;
  for (int i = 0; i < k; ++i) {
    cp_net* n = nets[i];
    if (!n || n->e->device != e->device) return fail(CP_E_ARG, "MAC batch member on another device");
    if (n->n >= 65536) return fail(CP_E_UNSUPPORTED, "MAC batch members need n < 65536");
    spec[i].net = n;
    spec[i].init = n->level_ptr(0);
    spec[i].levels = n->n + 3;
    const int nc = n_choice ? n_choice[i] : 0;
    if (nc < 0 || (nc > 0 && (!choice_var || !choice_val))) return fail(CP_E_ARG, "bad choice list");
    for (int j = 0; j < nc; ++j, ++c) {
      CP_TRY(check_var_val(n, choice_var[c], choice_val[c]));
      spec[i].choices.push_back(make_int2(choice_var[c], choice_val[c]));
    }
  }
  auto b = std::make_unique<cp_mac_batch>();
  CP_TRY(mac_start(e, spec, var_heuristic, time_limit_ms, b.get()));
  *out = b.release();
  return CP_OK;
}

int cp_mac_batch_poll(cp_mac_batch* b, uint8_t* done, cp_search_result* res, int* n_done) {
  if (!b || !done || !res) return fail(CP_E_ARG, "null argument");
  const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - b->t0).count();
  int nd = 0;
  for (int i = 0; i < b->k; ++i) {
    if (!b->reported[i]) {
      const volatile int* flag = &b->outs[i].done;
      if (*flag) {
        std::atomic_thread_fence(std::memory_order_acquire);
        const MacOut& o = b->outs[i];
        if (o.status < 0) return fail(o.status, "device MAC search failed (level stack or round limit)");
        cp_search_result r{};
        r.status = o.status;
        r.num_positive = o.npos;
        r.num_negative = o.nneg;
        r.propagations = o.props;
        r.solve_ms = ms;
        b->res[i] = r;
        b->reported[i] = 1;
      }
    }
    done[i] = b->reported[i];
    if (b->reported[i]) {
      res[i] = b->res[i];
      ++nd;
    }
  }
  if (nd < b->k) {
    const cudaError_t q = cudaEventQuery(b->ev);
    if (q != cudaSuccess && q != cudaErrorNotReady) return fail(CP_E_CUDA, std::string("MAC batch: ") + cudaGetErrorString(q));
    if (q == cudaSuccess) {
      // The launch has ended: results written meanwhile are collected, and
      // searches suspended at the end of their slice are resumed.
      bool again = false;
      for (int i = 0; i < b->k; ++i)
        if (!b->reported[i] && *reinterpret_cast<volatile int*>(&b->outs[i].done)) again = true;
      if (again) return cp_mac_batch_poll(b, done, res, n_done);
      CP_TRY(b->launch());
    }
  }
  if (n_done) *n_done = nd;
  return CP_OK;
}

int cp_mac_batch_wait(cp_mac_batch* b, cp_search_result* res) {
  if (!b) return fail(CP_E_ARG, "null batch");
  std::vector<uint8_t> done(b->k);
  std::vector<cp_search_result> tmp(b->k);
  int nd = 0;
  for (;;) {
    CP_CUDA(cudaEventSynchronize(b->ev));
    CP_TRY(cp_mac_batch_poll(b, done.data(), tmp.data(), &nd));  // relaunches suspended searches
    if (nd == b->k) break;
  }
  if (res)
    for (int i = 0; i < b->k; ++i) res[i] = tmp[i];
  return CP_OK;
}

int cp_mac_batch_solution(cp_mac_batch* b, int i, int* out) {
  if (!b || !out || i < 0 || i >= b->k) return fail(CP_E_ARG, "bad solution request");
  if (!b->reported[i]) return fail(CP_E_STATE, "search not finished");
  std::memcpy(out, b->sols + b->sol_off[i], static_cast<size_t>(b->n_of[i]) * sizeof(int));
  return CP_OK;
}

int cp_mac_batch_destroy(cp_mac_batch* b) {
  if (!b) return CP_OK;
  delete b;
  return CP_OK;
}

int cp_gsolver_solve(cp_net* net, int64_t time_limit_ms, cp_search_result* res, int* solution) {
  if (!net || !res || !solution) return fail(CP_E_ARG, "null argument");
  if (net->e->search_mode == 0 && !net->prefer_grid) {
    // The whole d-way search in one CTA, on the network's own level stack.
    std::vector<MacSpec> spec(1);
    spec[0].net = net;
    spec[0].init = net->level_ptr(0);
    spec[0].stack = net->d_levels;
    spec[0].levels = net->levels;
    cp_mac_batch b;
    CP_TRY(mac_start(net->e, spec, 2, time_limit_ms, &b));
    CP_TRY(cp_mac_batch_wait(&b, res));
    return cp_mac_batch_solution(&b, 0, solution);
  }
  DeviceGSolver g(net);
  return g.solve(time_limit_ms, res, solution);
}

// ---- generator --------------------------------------------------------
struct cp_instance {
  cpgen::Instance I;
};

int cp_gen_binary(int n, int d, int64_t e, double p_lo, double p_hi, double remove, uint64_t seed, cp_instance** out) {
  if (!out || n < 2 || d < 1 || e < 0) return fail(CP_E_ARG, "bad generator arguments");
  try {
    *out = new cp_instance{cpgen::random_binary(n, d, e, p_lo, p_hi, remove, seed)};
  } catch (const std::exception& ex) {
    return fail(CP_E_ARG, ex.what());
  }
  return CP_OK;
}

int cp_gen_mixed(int n, int d, int64_t e, double p_lo, double p_hi, int k3, int ntup, double remove, uint64_t seed,
                 cp_instance** out) {
  if (!out || n < 3 || d < 1 || e < 0 || k3 < 0 || ntup < 0) return fail(CP_E_ARG, "bad generator arguments");
  try {
    *out = new cp_instance{cpgen::random_mixed(n, d, e, p_lo, p_hi, k3, ntup, remove, seed)};
  } catch (const std::exception& ex) {
    return fail(CP_E_ARG, ex.what());
  }
  return CP_OK;
}

int cp_gen_uneven(uint64_t seed, int n_lo, int n_hi, int d_cap, cp_instance** out) {
  if (!out || n_lo < 2 || n_hi < n_lo || d_cap < 8) return fail(CP_E_ARG, "bad generator arguments");
  *out = new cp_instance{cpgen::uneven_instance(seed, n_lo, n_hi, d_cap)};
  return CP_OK;
}

int cp_gen_free(cp_instance* inst) {
  delete inst;
  return CP_OK;
}

int cp_gen_sizes(const cp_instance* inst, int64_t* sizes) {
  if (!inst || !sizes) return fail(CP_E_ARG, "null argument");
  const auto& I = inst->I;
  sizes[0] = I.n;
  sizes[1] = I.W;
  sizes[2] = I.n_bin();
  sizes[3] = I.n_tab();
  sizes[4] = static_cast<int64_t>(I.brows.size());
  sizes[5] = static_cast<int64_t>(I.tscope.size());
  sizes[6] = static_cast<int64_t>(I.ttup.size());
  sizes[7] = static_cast<int64_t>(cpgen::fingerprint(I));
  return CP_OK;
}

int cp_gen_export(const cp_instance* inst, int* dom, uint64_t* init, int* bin_scope, uint64_t* bin_rows, int* tab_arity,
                  int* tab_scope, int* tab_ntup, int* tab_tuples) {
  if (!inst) return fail(CP_E_ARG, "null instance");
  const auto& I = inst->I;
  if (dom) std::copy(I.dom.begin(), I.dom.end(), dom);
  if (init) std::copy(I.init.begin(), I.init.end(), init);
  if (bin_scope)
    for (int c = 0; c < I.n_bin(); ++c) {
      bin_scope[2 * c] = I.bx[c];
      bin_scope[2 * c + 1] = I.by[c];
    }
  if (bin_rows) std::copy(I.brows.begin(), I.brows.end(), bin_rows);
  if (tab_arity) std::copy(I.tarity.begin(), I.tarity.end(), tab_arity);
  if (tab_scope) std::copy(I.tscope.begin(), I.tscope.end(), tab_scope);
  if (tab_ntup) std::copy(I.tntup.begin(), I.tntup.end(), tab_ntup);
  if (tab_tuples) std::copy(I.ttup.begin(), I.ttup.end(), tab_tuples);
  return CP_OK;
}

// Seeded instances whose relation rows are generated on the device: the host
// draws the structure (scopes, tightness, removed values) from the same
// stream as cp_gen_binary / cp_gen_uneven, the rows come from relation_word
// on the GPU, so the network equals an upload of the host-generated one.
static int upload_generated(cp_engine* e, const cpgen::Instance& I, int max_levels, cp_net** out) {
  std::vector<int> scope(2 * static_cast<size_t>(I.n_bin()));
  for (int c = 0; c < I.n_bin(); ++c) {
    scope[2 * c] = I.bx[c];
    scope[2 * c + 1] = I.by[c];
  }
  cp_net* net = nullptr;
  CP_TRY(net_upload_impl(e, I.n, I.dom.data(), I.W, I.init.data(), I.n_bin(), scope.data(), nullptr, 0, nullptr,
                         nullptr, nullptr, nullptr, max_levels, &net, true));
  if (I.n_bin() > 0) {
    u64* d_seed = nullptr;
    u32* d_thr = nullptr;
    cudaError_t err = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&d_seed), I.bseed.size() * sizeof(u64),
                                              e->pool, e->stream);
    if (err == cudaSuccess)
      err = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&d_thr), I.bthr.size() * sizeof(u32), e->pool, e->stream);
    if (err == cudaSuccess)
      err = cudaMemcpyAsync(d_seed, I.bseed.data(), I.bseed.size() * sizeof(u64), cudaMemcpyHostToDevice, e->stream);
    if (err == cudaSuccess)
      err = cudaMemcpyAsync(d_thr, I.bthr.data(), I.bthr.size() * sizeof(u32), cudaMemcpyHostToDevice, e->stream);
    if (err == cudaSuccess)
      err = launch_gen_rows(net->dn, net->d_rel, net->d_bx, net->d_by, net->d_offA, d_seed, d_thr, e->stream);
    if (err == cudaSuccess)  // k_transpose writes every word of the B blocks
      err = launch_transpose(net->dn, net->d_rel, net->d_bx, net->d_by, net->d_offA, net->d_offB, e->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(e->stream);
    e->launches += 2;
    e->dev_free(d_seed);
    e->dev_free(d_thr);
    if (err != cudaSuccess) {
      cp_net_destroy(net);
      return fail(CP_E_CUDA, std::string("device generator: ") + cudaGetErrorString(err));
    }
  }
  *out = net;
  return CP_OK;
}

int cp_gen_binary_device(cp_engine* e, int n, int d, int64_t ne, double p_lo, double p_hi, double remove,
                         uint64_t seed, int max_levels, cp_net** out) {
  if (!e || !out || n < 2 || d < 1 || ne < 0) return fail(CP_E_ARG, "bad generator arguments");
  cpgen::Instance I;
  try {
    I = cpgen::random_binary(n, d, ne, p_lo, p_hi, remove, seed, false);
  } catch (const std::exception& ex) {
    return fail(CP_E_ARG, ex.what());
  }
  return upload_generated(e, I, max_levels, out);
}

int cp_gen_uneven_device(cp_engine* e, uint64_t seed, int n_lo, int n_hi, int d_cap, int max_levels, cp_net** out) {
  if (!e || !out || n_lo < 2 || n_hi < n_lo || d_cap < 8) return fail(CP_E_ARG, "bad generator arguments");
  const cpgen::Instance I = cpgen::uneven_instance(seed, n_lo, n_hi, d_cap, false);
  return upload_generated(e, I, max_levels, out);
}

int cp_net_rows_get(cp_net* net, uint64_t* out) {
  if (!net || !out) return fail(CP_E_ARG, "null argument");
  const int W = net->W_user, Wi = net->W;
  std::vector<u64> rows(static_cast<size_t>(net->relA_words));
  CP_TRY(d2h(net->e, rows.data(), net->d_rel, rows.size() * 8));
  int64_t src = 0, dst = 0;
  for (int c = 0; c < net->nb; ++c)
    for (int a = 0; a < net->dom[net->bx[c]]; ++a) {
      for (int w = 0; w < W; ++w) out[dst + w] = rows[src + w];
      src += Wi;
      dst += W;
    }
  return CP_OK;
}

int cp_net_upload_instance(cp_engine* e, const cp_instance* inst, int max_levels, cp_net** out) {
  if (!inst) return fail(CP_E_ARG, "null instance");
  const auto& I = inst->I;
  std::vector<int> scope(2 * static_cast<size_t>(I.n_bin()));
  for (int c = 0; c < I.n_bin(); ++c) {
    scope[2 * c] = I.bx[c];
    scope[2 * c + 1] = I.by[c];
  }
  return cp_net_upload(e, I.n, I.dom.data(), I.W, I.init.data(), I.n_bin(), scope.data(), I.brows.data(), I.n_tab(),
                       I.tarity.data(), I.tscope.data(), I.tntup.data(), I.ttup.data(), max_levels, out);
}

}  // extern "C"

// ===========================================================================
// Multi-instance batches
// ===========================================================================
namespace {

struct BatchGroup {
  int W = 1;
  bool tables = false;
  bool dense = false;  // members whose densest variable overflows a 100 KB tile
  std::vector<int> members;  // indices into cp_batch::nets
  BatchDev B;
  int max_n = 0;
  int slot_cap = 0;
  bool tiled = false;
  int tile_grid = 0;
  size_t cta_bytes = 0;
  bool cta_smem = true;
  void* gscratch = nullptr;
  size_t gstride = 0;
  int node_grid = 0;
  int sac_grid = 0;
  int sac_block = 256;
  int64_t total_values = 0;
  int64_t tiles_upper = 0;  // sum over members' variables of ceil(d / 32)
  int quota = 0;            // CTA quota of the sweep kernels (0: persistent grids)
  cudaGraphExec_t exec = nullptr;
  std::string key;  // autotuner cache key
};

std::string tune_cache_path() {
  const char* p = std::getenv("CPGPU_TUNE_CACHE");
  if (p && *p) return p;
  const char* h = std::getenv("HOME");
  return std::string(h && *h ? h : "/tmp") + "/.cache/cpgpu_tune.txt";
}

// Cache lines: "<key> <tiled> <sac_block>"; the last line of a key wins. The
// file is read once per path and kept in memory (batches are created per
// request tick by the server).
std::mutex g_tune_mu;
std::string g_tune_path;
std::map<std::string, std::pair<bool, int>> g_tune;

void tune_load_locked(const std::string& path) {
  if (path == g_tune_path) return;
  g_tune_path = path;
  g_tune.clear();
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return;
  char k[256];
  int t = 0, b = 0;
  while (std::fscanf(f, "%255s %d %d", k, &t, &b) == 3) g_tune[k] = {t != 0, b};
  std::fclose(f);
}

bool tune_lookup(const std::string& key, bool& tiled, int& block) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  tune_load_locked(tune_cache_path());
  auto it = g_tune.find(key);
  if (it == g_tune.end()) return false;
  tiled = it->second.first;
  block = it->second.second;
  return true;
}

void tune_store(const std::string& key, bool tiled, int block) {
  const std::string path = tune_cache_path();
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load_locked(path);
    g_tune[key] = {tiled, block};
  }
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) {
    const std::string dir = path.substr(0, slash);
    for (size_t i = 1; i <= dir.size(); ++i)
      if (i == dir.size() || dir[i] == '/') {
        const std::string sub = dir.substr(0, i);
        if (!sub.empty()) mkdir(sub.c_str(), 0755);
      }
  }
  FILE* f = std::fopen(path.c_str(), "a");
  if (!f) return;
  std::fprintf(f, "%s %d %d\n", key.c_str(), tiled ? 1 : 0, block);
  std::fclose(f);
}

}  // namespace

struct cp_batch {
  cp_engine* e = nullptr;
  int k = 0;
  std::vector<int> levels;  // working level of each member
  std::vector<cp_net*> nets;
  std::vector<std::pair<int, int>> where;  // member -> (group, index in the group)
  std::vector<int64_t> out_off;            // member -> word offset in a gathered domain buffer
  int64_t gather_words = 0;
  u64* d_gather = nullptr;
  int* d_edit = nullptr;  // member / var / val lists of cp_batch_load
  int64_t edit_cap = 0;
  std::vector<BatchGroup> groups;
  std::vector<void*> allocs;
  KStats* d_stats = nullptr;
  KStats* h_stats = nullptr;
  int* h_int = nullptr;
  bool use_graph = true;
  void* h_block = nullptr;  // pinned: h_stats, h_int
  ~cp_batch() {
    for (auto& g : groups)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    for (void* p : allocs) e->dev_free(p);
    e->pinned_put(h_block, 512);
  }
  template <typename T>
  int alloc(T** p, size_t count) {
    void* raw = nullptr;
    const size_t bytes = (std::max<size_t>(count * sizeof(T), 16) + 255) & ~size_t(255);
    CP_TRY(e->dev_alloc(&raw, bytes + 256));
    allocs.push_back(raw);
    *p = reinterpret_cast<T*>((reinterpret_cast<uintptr_t>(raw) + 255) & ~uintptr_t(255));
    return CP_OK;
  }
};

namespace {

int batch_group_setup(cp_batch* b, BatchGroup& g) {
  cp_engine* e = b->e;
  cudaStream_t s = e->stream;
  const int kg = static_cast<int>(g.members.size());
  std::vector<DevNet> nets(kg);
  std::vector<u64*> roots(kg), bases(kg);
  std::vector<int64_t> offs(kg), woff(kg);
  std::vector<int> wuser(kg);
  int64_t weak_words = 0;
  std::vector<int> var_base(kg + 1, 0);
  int max_deg = 1;
  g.cta_bytes = 0;
  g.total_values = 0;
  for (int i = 0; i < kg; ++i) {
    cp_net* n = b->nets[g.members[i]];
    nets[i] = n->dn;
    roots[i] = n->level_ptr(b->levels[g.members[i]]);
    bases[i] = n->d_levels;
    offs[i] = b->out_off[g.members[i]];
    wuser[i] = n->W_user;
    woff[i] = weak_words;
    weak_words += static_cast<int64_t>(2) * n->nb * kWeakStride;
    var_base[i + 1] = var_base[i] + n->n;
    g.max_n = std::max(g.max_n, n->n);
    g.cta_bytes = std::max(g.cta_bytes, cta_state_bytes(n->dn));
    g.total_values += n->dn.total_values;
    for (int d : n->dom) g.tiles_upper += (d + 31) / 32;
    max_deg = std::max(max_deg, n->max_deg);
  }
  const int tv = var_base[kg];
  std::vector<int> var_inst(tv);
  for (int i = 0; i < kg; ++i)
    for (int x = var_base[i]; x < var_base[i + 1]; ++x) var_inst[x] = i;
  BatchDev& B = g.B;
  B.k = kg;
  B.total_vars = tv;
  // Member descriptors: one device block, one copy from pinned staging.
  DevNet* d_nets;
  u64** d_roots;
  u64** d_bases;
  int64_t* d_offs;
  int64_t* d_woff;
  int *d_vb, *d_vi, *d_wu;
  MetaPack mp;
  mp.add(&d_nets, nets.data(), kg);
  mp.add(&d_roots, roots.data(), kg);
  mp.add(&d_bases, bases.data(), kg);
  mp.add(&d_offs, offs.data(), kg);
  mp.add(&d_woff, woff.data(), kg);
  mp.add(&d_wu, wuser.data(), kg);
  mp.add(&d_vb, var_base.data(), kg + 1);
  mp.add(&d_vi, var_inst.data(), tv);
  char* d_meta = nullptr;
  CP_TRY(b->alloc(&d_meta, mp.total));
  PinnedLease stage(e);
  CP_TRY(stage.get(mp.total));
  for (const auto& q : mp.parts) {
    if (q.bytes) std::memcpy(static_cast<char*>(stage.p) + q.off, q.src, q.bytes);
    *q.dst = d_meta + q.off;
  }
  CP_CUDA(cudaMemcpyAsync(d_meta, stage.p, mp.total, cudaMemcpyHostToDevice, s));
  B.nets = d_nets;
  B.roots = d_roots;
  B.bases = d_bases;
  B.out_off = d_offs;
  B.weak_off = d_woff;
  B.weak = nullptr;
  B.snap = nullptr;
  if (!g.tables && weak_words > 0) {
    CP_TRY(b->alloc(&B.weak, static_cast<size_t>(weak_words)));
    CP_TRY(b->alloc(&B.snap, static_cast<size_t>(tv) * g.W));
  }
  B.wuser = d_wu;
  B.var_base = d_vb;
  B.var_inst = d_vi;
  CP_TRY(b->alloc(&B.inc, kg));
  CP_TRY(b->alloc(&B.act, kg));
  CP_TRY(b->alloc(&B.removed, kg));
  CP_TRY(b->alloc(&B.evt, tv));
  CP_TRY(b->alloc(&B.nevt, kg));
  CP_TRY(b->alloc(&B.evt_fb, (tv + 31) / 32));
  CP_TRY(b->alloc(&B.act_list, kg));
  CP_TRY(b->alloc(&B.nact, 4));
  CP_TRY(b->alloc(&B.work, g.total_values));
  CP_TRY(b->alloc(&B.nwork, 4));
  CP_TRY(b->alloc(&B.ok, g.total_values));
  CP_TRY(b->alloc(&B.cursor, 4));
  CP_TRY(b->alloc(&B.tiles, static_cast<size_t>(tv) * 2 * g.W));
  CP_TRY(b->alloc(&B.ntiles, 4));
  CP_TRY(b->alloc(&B.tcursor, 4));
  CP_TRY(b->alloc(&B.deep, g.total_values));
  CP_TRY(b->alloc(&B.ndeep, 4));
  // CTA-local state: shared memory when it fits.
  g.cta_smem = g.cta_bytes + 2048 <= e->smem_optin;
  // Per-CTA global scratch is indexed by CTA: quotas need shared-memory state.
  g.quota = g.cta_smem ? e->cta_quota : 0;
  const size_t smem = g.cta_smem ? g.cta_bytes : 0;
  int per_sm_node = batch_node_blocks_per_sm(g.W, g.tables, e->block_node, smem);
  int per_sm_sac = batch_sac_blocks_per_sm(g.W, g.tables, g.sac_block, smem);
  if (per_sm_node < 1 || per_sm_sac < 1) return fail(CP_E_UNSUPPORTED, "batch kernels do not fit on an SM");
  if (e->ctas_per_sm > 0) per_sm_sac = std::min(per_sm_sac, e->ctas_per_sm);
  g.node_grid = std::min(per_sm_node * e->sm_count, std::max(1, kg));
  g.sac_grid = per_sm_sac * e->sm_count;
  if (!g.cta_smem) {
    g.gstride = (g.cta_bytes + 255) & ~size_t(255);
    char* p;
    CP_TRY(b->alloc(&p, g.gstride * static_cast<size_t>(std::max(g.node_grid, g.sac_grid))));
    g.gscratch = p;
  }
  // Tiled sweep where the network kind allows it.
  g.tiled = false;
  g.tile_grid = 0;
  if (!g.tables && g.max_n < 65536) {
    const size_t per_slot = static_cast<size_t>(32) * g.W * 8 + 16;  // domains + neighbour record
    const size_t optin = e->smem_optin > 4096 ? e->smem_optin - 4096 : 0;
    const size_t need = static_cast<size_t>(g.max_n) * 4 + per_slot * static_cast<size_t>(max_deg);
    const size_t budget = std::min<size_t>(optin, g.dense ? need : 100 * 1024);
    if (static_cast<size_t>(g.max_n) * 4 + per_slot * 8 <= budget) {
      g.slot_cap = static_cast<int>(std::min<size_t>(max_deg, (budget - static_cast<size_t>(g.max_n) * 4) / per_slot));
      const int per_sm_t = batch_tile_blocks_per_sm(g.W, g.slot_cap, g.max_n);
      if (per_sm_t > 0) {
        g.tile_grid = per_sm_t * e->sm_count;
        g.tiled = true;
      }
    }
  }
  // Autotuner cache: shape bucket of the group.
  int maxd = 0;
  for (int m : g.members)
    for (int d : b->nets[m]->dom) maxd = std::max(maxd, d);
  char key[160];
  std::snprintf(key, sizeof key, "W%d_tab%d_n%d_deg%d_d%d_k%d", g.W, g.tables ? 1 : 0, 1 << (32 - __builtin_clz(std::max(1, g.max_n))),
                1 << (32 - __builtin_clz(std::max(1, max_deg))), maxd, 1 << (32 - __builtin_clz(std::max(1, kg))));
  g.key = key;
  bool t_tiled = g.tiled;
  int t_block = g.sac_block;
  if (tune_lookup(g.key, t_tiled, t_block)) {
    g.tiled = g.tiled && t_tiled;
    if (t_block == 128 || t_block == 256) g.sac_block = t_block;
  }
  CP_CUDA(cudaStreamSynchronize(s));
  return CP_OK;
}

// One sweep of a group: reset counters, build pairs/tiles, test, commit,
// select the instances with removals, propagate their removals.
int batch_sweep_launches(cp_batch* b, BatchGroup& g, bool with_commit) {
  cp_engine* e = b->e;
  cudaStream_t s = e->stream;
  BatchDev& B = g.B;
  const int kg = B.k;
  CP_CUDA(cudaMemsetAsync(B.nwork, 0, sizeof(int), s));
  CP_CUDA(cudaMemsetAsync(B.cursor, 0, sizeof(int), s));
  CP_CUDA(cudaMemsetAsync(B.ntiles, 0, sizeof(int), s));
  CP_CUDA(cudaMemsetAsync(B.tcursor, 0, sizeof(int), s));
  CP_CUDA(cudaMemsetAsync(B.ndeep, 0, sizeof(int), s));
  CP_CUDA(cudaMemsetAsync(B.removed, 0, kg * sizeof(int), s));
  CP_CUDA(cudaMemsetAsync(B.nevt, 0, kg * sizeof(int), s));
  CP_CUDA(cudaMemsetAsync(B.evt_fb, 0, ((B.total_vars + 31) / 32) * sizeof(u32), s));
  const size_t smem = g.cta_smem ? g.cta_bytes : 0;
  CP_CUDA(launch_batch_build(g.W, B, g.tiled, s));
  // With a CTA quota the grids cover every tile / branch (upper bounds); CTAs
  // past the actual count retire at once.
  const int q = g.quota;
  auto cover = [&](int64_t units, int persistent) {
    return q > 0 ? static_cast<int>(std::min<int64_t>((units + q - 1) / q, int64_t(1) << 30)) : persistent;
  };
  if (B.snap) {
    // Sweep-start domains (early removals then change only the roots).
    CP_CUDA(launch_batch_snap(g.W, B, s));
    e->launches += 1;
  }
  if (g.tiled) {
    if (B.weak) {
      CP_CUDA(launch_batch_weak(g.W, B, s));
      e->launches += 1;
    }
    CP_CUDA(launch_batch_tile(g.W, B, g.slot_cap, g.max_n, b->d_stats, cover(g.tiles_upper, g.tile_grid), q, s));
    CP_CUDA(launch_batch_sac(g.W, g.tables, B, true, b->d_stats, g.sac_block, cover(g.total_values, g.sac_grid), smem,
                             g.gscratch, g.gstride, q, s));
  } else {
    CP_CUDA(launch_batch_sac(g.W, g.tables, B, false, b->d_stats, g.sac_block, cover(g.total_values, g.sac_grid), smem,
                             g.gscratch, g.gstride, q, s));
  }
  e->launches += g.tiled ? 3 : 2;
  if (with_commit) {
    CP_CUDA(launch_batch_commit(g.W, B, b->d_stats, s));
    CP_CUDA(cudaMemsetAsync(B.nact, 0, sizeof(int), s));
    CP_CUDA(launch_batch_select(B, false, s));
    CP_CUDA(launch_batch_node(g.W, g.tables, B, kOpEvents, b->d_stats, e->block_node, g.node_grid, smem, g.gscratch,
                              g.gstride, s));
    e->launches += 3;
  }
  return CP_OK;
}

int batch_root(cp_batch* b, BatchGroup& g) {
  cp_engine* e = b->e;
  cudaStream_t s = e->stream;
  BatchDev& B = g.B;
  const size_t smem = g.cta_smem ? g.cta_bytes : 0;
  CP_CUDA(cudaMemsetAsync(B.inc, 0, B.k, s));
  CP_CUDA(cudaMemsetAsync(B.removed, 0, B.k * sizeof(int), s));
  CP_CUDA(cudaMemsetAsync(B.nact, 0, sizeof(int), s));
  CP_CUDA(launch_batch_select(B, true, s));
  CP_CUDA(launch_batch_node(g.W, g.tables, B, kOpRoot, b->d_stats, e->block_node, g.node_grid, smem, g.gscratch,
                            g.gstride, s));
  CP_CUDA(cudaMemsetAsync(B.nact, 0, sizeof(int), s));
  CP_CUDA(launch_batch_select(B, true, s));
  e->launches += 3;
  return CP_OK;
}

int batch_stats_begin(cp_batch* b) {
  KStats z{};
  z.fail_var = -1;
  *b->h_stats = z;
  CP_CUDA(cudaMemcpyAsync(b->d_stats, b->h_stats, sizeof(KStats), cudaMemcpyHostToDevice, b->e->stream));
  return CP_OK;
}

int batch_read_int(cp_batch* b, const int* d) {
  CP_CUDA(cudaMemcpyAsync(b->h_int, d, sizeof(int), cudaMemcpyDeviceToHost, b->e->stream));
  CP_CUDA(cudaStreamSynchronize(b->e->stream));
  return CP_OK;
}

int batch_finish(cp_batch* b, cp_stats* st, uint8_t* inconsistent, int sweeps, int launches) {
  cp_engine* e = b->e;
  CP_CUDA(cudaEventRecord(e->ev1, e->stream));
  CP_CUDA(cudaMemcpyAsync(b->h_stats, b->d_stats, sizeof(KStats), cudaMemcpyDeviceToHost, e->stream));
  CP_CUDA(cudaStreamSynchronize(e->stream));
  if (b->h_stats->error) return fail(b->h_stats->error, "device-side check failed in a batch");
  if (inconsistent) {
    for (auto& g : b->groups) {
      std::vector<uint8_t> inc(g.B.k);
      CP_TRY(d2h(e, inc.data(), g.B.inc, g.B.k));
      for (int i = 0; i < g.B.k; ++i) inconsistent[g.members[i]] = inc[i];
    }
  }
  if (st) {
    const KStats& k = *b->h_stats;
    cp_stats s{};
    s.revisions = static_cast<int64_t>(k.revisions);
    s.rows = static_cast<int64_t>(k.rows + k.tuples);
    s.fixpoints = static_cast<int64_t>(k.fixpoints);
    s.branches = static_cast<int64_t>(k.branches);
    s.deletions = static_cast<int64_t>(k.removed);
    s.rounds = k.rounds_max;
    s.sweeps = sweeps;
    s.launches = launches;
    s.device_ms = elapsed_ms(e);
    int ninc = 0;
    for (auto& g : b->groups) {
      std::vector<uint8_t> inc(g.B.k);
      CP_TRY(d2h(e, inc.data(), g.B.inc, g.B.k));
      for (uint8_t v : inc) ninc += v;
    }
    s.inconsistent = ninc;
    *st = s;
  }
  return CP_OK;
}

}  // namespace

extern "C" {

int cp_batch_create(cp_engine* e, int k, cp_net* const* nets, int level, cp_batch** out) {
  if (k < 1 || k >= 32768) return fail(CP_E_UNSUPPORTED, "a batch holds 1 to 32767 instances");
  std::vector<int> levels(static_cast<size_t>(k), level);
  return cp_batch_create_levels(e, k, nets, levels.data(), out);
}

int cp_batch_create_levels(cp_engine* e, int k, cp_net* const* nets, const int* levels, cp_batch** out) {
  if (!e || !out || k < 1 || !nets || !levels) return fail(CP_E_ARG, "bad batch arguments");
  if (k >= 32768) return fail(CP_E_UNSUPPORTED, "at most 32767 instances per batch");
  CP_CUDA(cudaSetDevice(e->device));
  auto b = std::make_unique<cp_batch>();
  b->e = e;
  b->k = k;
  b->levels.assign(levels, levels + k);
  b->nets.assign(nets, nets + k);
  b->out_off.resize(k);
  std::vector<std::pair<const cp_net*, int>> seen;
  for (int i = 0; i < k; ++i) {
    // Members may live on another engine of the same device: the batch only
    // reads their relations and writes their working levels, in the batch
    // engine's stream order; the caller keeps other users off those levels.
    if (!nets[i] || nets[i]->e->device != e->device) return fail(CP_E_ARG, "batch member on another device");
    if (nets[i]->n >= 65536) return fail(CP_E_UNSUPPORTED, "batch members need n < 65536");
    if (levels[i] < 0 || levels[i] >= nets[i]->levels) return fail(CP_E_ARG, "level out of range for a batch member");
    seen.emplace_back(nets[i], levels[i]);
    b->out_off[i] = b->gather_words;
    b->gather_words += static_cast<int64_t>(nets[i]->n) * nets[i]->W_user;
  }
  std::sort(seen.begin(), seen.end());
  if (std::adjacent_find(seen.begin(), seen.end()) != seen.end())
    return fail(CP_E_ARG, "two batch members share a network level");
  for (int i = 0; i < k; ++i) {
    const int W = nets[i]->W;
    const bool tab = nets[i]->nt > 0;
    // Members whose densest variable does not fit a 100 KB tile form their
    // own group, whose tiles get the larger shared-memory budget.
    const bool dense = !tab && static_cast<size_t>(nets[i]->n) * 4 +
                                       static_cast<size_t>(32) * W * 8 * nets[i]->max_deg > 100 * 1024;
    BatchGroup* g = nullptr;
    for (auto& gg : b->groups)
      if (gg.W == W && gg.tables == tab && gg.dense == dense) g = &gg;
    if (!g) {
      b->groups.emplace_back();
      g = &b->groups.back();
      g->W = W;
      g->tables = tab;
      g->dense = dense;
    }
    g->members.push_back(i);
  }
  b->where.resize(k);
  for (size_t gi = 0; gi < b->groups.size(); ++gi)
    for (size_t j = 0; j < b->groups[gi].members.size(); ++j)
      b->where[b->groups[gi].members[j]] = {static_cast<int>(gi), static_cast<int>(j)};
  static_assert(sizeof(KStats) <= 256, "batch pinned block layout");
  CP_TRY(e->pinned_get(512, &b->h_block));
  b->h_stats = static_cast<KStats*>(b->h_block);
  b->h_int = reinterpret_cast<int*>(static_cast<char*>(b->h_block) + 256);
  CP_TRY(b->alloc(&b->d_stats, 1));
  for (auto& g : b->groups) CP_TRY(batch_group_setup(b.get(), g));
  ++e->live_nets;
  *out = b.release();
  return CP_OK;
}

int cp_batch_destroy(cp_batch* b) {
  if (!b) return CP_OK;
  cp_engine* e = b->e;
  cudaStreamSynchronize(e->stream);
  delete b;
  --e->live_nets;  // a batch holds the engine like a network does
  if (e->closed && e->live_nets == 0) engine_free(e);
  return CP_OK;
}

int cp_batch_set_graphs(cp_batch* b, int use_graphs) {
  if (!b) return fail(CP_E_ARG, "null batch");
  b->use_graph = use_graphs != 0;
  return CP_OK;
}

int cp_batch_ac(cp_batch* b, cp_stats* st, uint8_t* inconsistent) {
  if (!b) return fail(CP_E_ARG, "null batch");
  cp_engine* e = b->e;
  CP_TRY(batch_stats_begin(b));
  CP_CUDA(cudaEventRecord(e->ev0, e->stream));
  int launches = 0;
  for (auto& g : b->groups) {
    CP_TRY(batch_root(b, g));
    launches += 3;
  }
  return batch_finish(b, st, inconsistent, 0, launches);
}

int cp_batch_sac1(cp_batch* b, cp_stats* st, uint8_t* inconsistent) {
  if (!b) return fail(CP_E_ARG, "null batch");
  cp_engine* e = b->e;
  cudaStream_t s = e->stream;
  CP_TRY(batch_stats_begin(b));
  CP_CUDA(cudaEventRecord(e->ev0, s));
  int launches = 0, max_sweeps = 0;
  for (auto& g : b->groups) {
    CP_TRY(batch_root(b, g));
    launches += 3;
    if (b->use_graph && !g.exec) {
      // Capture one sweep of this group; it is replayed until no instance
      // changes (the grids are persistent, all counts are read on device).
      cudaGraph_t graph;
      CP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      const int64_t l0 = e->launches;
      int rc = batch_sweep_launches(b, g, true);
      e->launches = l0;
      cudaError_t ce = cudaStreamEndCapture(s, &graph);
      if (rc != CP_OK) return rc;
      CP_CUDA(ce);
      CP_CUDA(cudaGraphInstantiate(&g.exec, graph, 0));
      cudaGraphDestroy(graph);
    }
    int sweeps = 0;
    for (;;) {
      ++sweeps;
      if (b->use_graph) {
        CP_CUDA(cudaGraphLaunch(g.exec, s));
        e->launches += g.tiled ? 6 : 5;
      } else {
        CP_TRY(batch_sweep_launches(b, g, true));
      }
      launches += g.tiled ? 6 : 5;
      CP_TRY(batch_read_int(b, g.B.nact));
      if (*b->h_int == 0) break;
    }
    max_sweeps = std::max(max_sweeps, sweeps);
  }
  return batch_finish(b, st, inconsistent, max_sweeps, launches);
}

// Times one sweep (without committing) of each group with the tiled and the
// general kernel and with 128- and 256-thread general CTAs, keeps the fastest
// and records it in the tuning cache ($CPGPU_TUNE_CACHE, default
// ~/.cache/cpgpu_tune.txt) under the group's shape key.
int cp_batch_tune(cp_batch* b) {
  if (!b) return fail(CP_E_ARG, "null batch");
  cp_engine* e = b->e;
  cudaStream_t s = e->stream;
  for (auto& g : b->groups) {
    CP_TRY(batch_stats_begin(b));
    CP_TRY(batch_root(b, g));
    // Trial sweeps only test: no early removals from the members' domains.
    u64* snap = g.B.snap;
    g.B.snap = nullptr;
    const bool can_tile = g.tile_grid > 0;
    struct Cand {
      bool tiled;
      int block;
    };
    std::vector<Cand> cands = {{false, 256}, {false, 128}};
    if (can_tile) cands.insert(cands.begin(), Cand{true, 256});
    float best = 1e30f;
    Cand pick = cands[0];
    for (const Cand& c : cands) {
      g.tiled = c.tiled;
      g.sac_block = c.block;
      float ms_best = 1e30f;
      for (int rep = 0; rep < 2; ++rep) {
        CP_CUDA(cudaEventRecord(e->ev0, s));
        CP_TRY(batch_sweep_launches(b, g, false));
        CP_CUDA(cudaEventRecord(e->ev1, s));
        CP_CUDA(cudaEventSynchronize(e->ev1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e->ev0, e->ev1);
        ms_best = std::min(ms_best, ms);
      }
      if (ms_best < best) {
        best = ms_best;
        pick = c;
      }
    }
    g.B.snap = snap;
    g.tiled = pick.tiled;
    g.sac_block = pick.block;
    if (g.exec) {
      cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
    }
    tune_store(g.key, g.tiled, g.sac_block);
  }
  return CP_OK;
}

int cp_batch_copy_level(cp_batch* b, int src) { return cp_batch_load(b, src, 0, nullptr, nullptr, nullptr); }

int cp_batch_load(cp_batch* b, int src_level, int n_edit, const int* member, const int* var, const int* val) {
  if (!b) return fail(CP_E_ARG, "null batch");
  if (n_edit < 0 || (n_edit > 0 && (!member || !var || !val))) return fail(CP_E_ARG, "bad edit list");
  for (cp_net* n : b->nets)
    if (src_level < 0 || src_level >= n->levels) return fail(CP_E_ARG, "source level out of range for a batch member");
  for (int j = 0; j < n_edit; ++j) {
    if (member[j] < 0 || member[j] >= b->k) return fail(CP_E_ARG, "edit member out of range");
    CP_TRY(check_var_val(b->nets[member[j]], var[j], val[j]));
  }
  cp_engine* e = b->e;
  cudaStream_t s = e->stream;
  for (auto& g : b->groups) {
    CP_CUDA(launch_batch_copy(g.W, g.B, src_level, s));
    ++e->launches;
  }
  if (n_edit > 0) {
    if (n_edit > b->edit_cap) {  // a smaller earlier list buffer stays until the batch goes
      b->edit_cap = std::max<int64_t>(n_edit, 2 * b->edit_cap);
      CP_TRY(b->alloc(&b->d_edit, 3 * static_cast<size_t>(b->edit_cap)));
    }
    // Edits ordered by group: [member in group | var | val] per group.
    const int ng = static_cast<int>(b->groups.size());
    std::vector<int> cnt(ng + 1, 0);
    for (int j = 0; j < n_edit; ++j) ++cnt[b->where[member[j]].first + 1];
    for (int gi = 0; gi < ng; ++gi) cnt[gi + 1] += cnt[gi];
    PinnedLease stage(e);
    CP_TRY(stage.get(3 * sizeof(int) * static_cast<size_t>(n_edit)));
    int* h = static_cast<int*>(stage.p);
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int j = 0; j < n_edit; ++j) {
      const auto& w = b->where[member[j]];
      const int at = fill[w.first]++;
      h[at] = w.second;
      h[n_edit + at] = var[j];
      h[2 * n_edit + at] = val[j];
    }
    CP_CUDA(cudaMemcpyAsync(b->d_edit, h, 3 * sizeof(int) * static_cast<size_t>(n_edit), cudaMemcpyHostToDevice, s));
    for (int gi = 0; gi < ng; ++gi) {
      const int c = cnt[gi + 1] - cnt[gi];
      if (c == 0) continue;
      const int o = cnt[gi];
      CP_CUDA(launch_batch_edit(b->groups[gi].W, b->groups[gi].B, c, b->d_edit + o, b->d_edit + n_edit + o,
                                b->d_edit + 2 * n_edit + o, s));
      ++e->launches;
    }
  }
  CP_CUDA(cudaStreamSynchronize(s));
  return CP_OK;
}

int cp_batch_dom_get(cp_batch* b, uint64_t* out) {
  if (!b || !out) return fail(CP_E_ARG, "null argument");
  cp_engine* e = b->e;
  if (!b->d_gather) CP_TRY(b->alloc(&b->d_gather, static_cast<size_t>(std::max<int64_t>(1, b->gather_words))));
  for (auto& g : b->groups) {
    CP_CUDA(launch_batch_gather(g.W, g.B, b->d_gather, e->stream));
    ++e->launches;
  }
  CP_TRY(d2h(e, out, b->d_gather, static_cast<size_t>(b->gather_words) * 8));
  return CP_OK;
}

int cp_batch_info(const cp_batch* b, int group, int* info) {
  if (!b || !info || group < 0 || group >= static_cast<int>(b->groups.size()))
    return fail(CP_E_ARG, "bad batch info arguments");
  const BatchGroup& g = b->groups[group];
  info[0] = static_cast<int>(b->groups.size());
  info[1] = g.W;
  info[2] = g.tables ? 1 : 0;
  info[3] = static_cast<int>(g.members.size());
  info[4] = g.tiled ? 1 : 0;
  info[5] = g.sac_block;
  info[6] = g.slot_cap;
  info[7] = g.cta_smem ? 1 : 0;
  return CP_OK;
}

}  // extern "C"
