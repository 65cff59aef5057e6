// cp_enforce_ac_static: the AC fixpoint of a binary network held entirely in
// the caller's device memory, computed without allocating anything.
//
// Who needs it: callers that must not call cudaMalloc or cudaFree while they
// run. cudaMalloc and cudaFree synchronise the whole device, which stalls a
// latency-bound serving or search loop, and a host framework that already
// owns the device's memory budget (a caching allocator that has reserved it,
// or a plugin host that hands its plugins preallocated buffers) may not let a
// plugin allocate at all. Such callers keep the network and domains in their
// own device buffers and pass them in; every scratch structure the kernels
// need lives in one static device array of this file.
//
// Limits: n <= 2048 variables, W <= 2 words per domain (at most 128 values),
// at most 2048 binary constraints. The static array is kStaticScratchBytes
// (9 MiB) on every GPU where the library is loaded, held until the process
// exits. All calls on a device share it and it keeps the last call's
// contents: each call clears what must start at zero, and calls whose work
// overlaps on the GPU (different streams, or other host threads) race on it.
// The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture begins. The address is kept for the life of the
// device's current context: a call that finds another context current (the
// primary context was reset and re-created) looks it up again.
#include <cuda.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/cpgpu.h"
#include "cp_internal.h"

namespace cpgpu {
namespace {

constexpr int kStaticMaxVars = 2048;
constexpr int kStaticMaxWords = 2;
constexpr int kStaticMaxBin = 2048;
constexpr int kStaticChunk = 8;
constexpr size_t kStaticScratchBytes = size_t(9) << 20;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];


// Byte offsets of the scratch regions for one call (worst case of the limits
// above; independent of the actual domain sizes).
struct StaticLayout {
  size_t arc_start, fill, tinc, bx, by, offA, offB, arcs, stats, rel, cta, total;
};

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

StaticLayout static_layout(int n, int W, int nb, size_t cta_bytes) {
  StaticLayout L;
  size_t o = 0;
  L.arc_start = o; o = up256(o + (size_t(n) + 1) * 4);
  L.fill = o;      o = up256(o + size_t(n) * 4);
  L.tinc = o;      o = up256(o + (size_t(n) + 1) * 4);
  L.bx = o;        o = up256(o + size_t(nb) * 4 + 4);
  L.by = o;        o = up256(o + size_t(nb) * 4 + 4);
  L.offA = o;      o = up256(o + size_t(nb) * 8 + 8);
  L.offB = o;      o = up256(o + size_t(nb) * 8 + 8);
  L.arcs = o;      o = up256(o + size_t(2) * nb * sizeof(Arc) + sizeof(Arc));
  L.stats = o;     o = up256(o + sizeof(KStats));
  L.rel = o;       o = up256(o + size_t(2) * nb * (64 * W) * W * 8);
  L.cta = o;       o = up256(o + cta_bytes);
  L.total = o;
  return L;
}

// Exclusive prefix sum over value(0..m-1) by the whole CTA (blockDim.x a
// multiple of 32, at most 1024): out[i] = value(0) + ... + value(i-1).
// Returns the total to every thread; ends with the CTA synchronised.
template <typename T, typename F>
__device__ T cta_exclusive_scan(int m, F value, T* out) {
  __shared__ T s_warp[32];
  __shared__ T s_carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) s_carry = T(0);
  __syncthreads();
  for (int base = 0; base < m; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const T v = i < m ? value(i) : T(0);
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
      T w = lane < nw ? s_warp[lane] : T(0);
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      s_warp[lane] = w;
    }
    __syncthreads();
    const T carry = s_carry;
    if (i < m) out[i] = carry + (warp ? s_warp[warp - 1] : T(0)) + x - v;
    __syncthreads();
    if (threadIdx.x == 0) s_carry = carry + s_warp[nw - 1];
    __syncthreads();
  }
  // Every thread reads the total before the next scan may reset s_carry.
  const T total = s_carry;
  __syncthreads();
  return total;
}

// One CTA: validates the inputs, zeroes the counters, and builds the arc
// incidence lists, relation offsets and A blocks in the scratch array.
__global__ void k_static_prep(int n, int W, int nb, const int* dsize, const int* scope, const u64* rows, u64* dom,
                              unsigned char* scratch, StaticLayout L) {
  int* arc_start = reinterpret_cast<int*>(scratch + L.arc_start);
  int* fill = reinterpret_cast<int*>(scratch + L.fill);
  int* tinc = reinterpret_cast<int*>(scratch + L.tinc);
  int* bx = reinterpret_cast<int*>(scratch + L.bx);
  int* by = reinterpret_cast<int*>(scratch + L.by);
  int64_t* offA = reinterpret_cast<int64_t*>(scratch + L.offA);
  int64_t* offB = reinterpret_cast<int64_t*>(scratch + L.offB);
  Arc* arcs = reinterpret_cast<Arc*>(scratch + L.arcs);
  KStats* st = reinterpret_cast<KStats*>(scratch + L.stats);
  u64* rel = reinterpret_cast<u64*>(scratch + L.rel);
  __shared__ int s_bad;
  if (threadIdx.x == 0) {
    s_bad = 0;
    *st = KStats{};
    st->fail_var = -1;
  }
  for (int i = threadIdx.x; i <= n; i += blockDim.x) {
    arc_start[i] = 0;
    tinc[i] = 0;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) fill[i] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    if (dsize[i] < 1 || dsize[i] > 64 * W) atomicExch(&s_bad, 1);
  for (int c = threadIdx.x; c < nb; c += blockDim.x) {
    const int x = scope[2 * c], y = scope[2 * c + 1];
    if (x < 0 || x >= n || y < 0 || y >= n || x == y) {
      atomicExch(&s_bad, 1);
    } else {
      bx[c] = x;
      by[c] = y;
      atomicAdd(&fill[x], 1);
      atomicAdd(&fill[y], 1);
    }
  }
  __syncthreads();
  if (s_bad) {
    // Leave an empty incidence structure so that the fixpoint kernel reads
    // nothing, and report the bad input.
    for (int i = threadIdx.x; i <= n; i += blockDim.x) arc_start[i] = 0;
    if (threadIdx.x == 0) st->error = CP_E_ARG;
    return;
  }
  // Incidence offsets and relation block offsets (A blocks of all
  // constraints, then B blocks) by CTA-wide scans.
  const int incidences = cta_exclusive_scan<int>(n, [&](int i) { return fill[i]; }, arc_start);
  if (threadIdx.x == 0) arc_start[n] = incidences;
  for (int i = threadIdx.x; i < n; i += blockDim.x) fill[i] = 0;
  const int64_t a_words =
      cta_exclusive_scan<int64_t>(nb, [&](int c) { return int64_t(dsize[bx[c]]) * W; }, offA);
  cta_exclusive_scan<int64_t>(nb, [&](int c) { return int64_t(dsize[by[c]]) * W; }, offB);
  for (int c = threadIdx.x; c < nb; c += blockDim.x) offB[c] += a_words;
  __syncthreads();
  for (int c = threadIdx.x; c < nb; c += blockDim.x) {
    const int x = bx[c], y = by[c];
    arcs[arc_start[y] + atomicAdd(&fill[y], 1)] = Arc{x, static_cast<u32>(offA[c]), static_cast<u32>(offB[c]), y};
    arcs[arc_start[x] + atomicAdd(&fill[x], 1)] = Arc{y, static_cast<u32>(offB[c]), static_cast<u32>(offA[c]), x};
  }
  // A blocks are the caller's rows in constraint order; B blocks start zeroed.
  const int64_t b_end = nb ? offB[nb - 1] + int64_t(dsize[by[nb - 1]]) * W : 0;
  for (int64_t i = threadIdx.x; i < a_words; i += blockDim.x) rel[i] = rows[i];
  for (int64_t i = a_words + threadIdx.x; i < b_end; i += blockDim.x) rel[i] = 0ull;
  // Domain bits at or beyond a variable's size are cleared (the kernels index
  // support rows by live values).
  for (int x = threadIdx.x; x < n; x += blockDim.x)
    for (int w = 0; w < W; ++w) {
      const int lo = w * 64, d = dsize[x];
      if (d - lo < 64) dom[size_t(x) * W + w] &= (d - lo <= 0) ? 0ull : ((1ull << (d - lo)) - 1ull);
    }
  __syncthreads();
  // B blocks: one warp per (constraint, group of 32 x values); lane l holds
  // the row of x = 32g + l, and the ballot over lanes of bit b is the 32-bit
  // slice of y=b's row.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int groups = 2 * W;
  for (int item = warp; item < nb * groups; item += nwarps) {
    const int c = item / groups, g = item % groups;
    const int dx = dsize[bx[c]], dy = dsize[by[c]];
    if (g * 32 >= dx) continue;
    const int a = g * 32 + lane;
    u64 row[kStaticMaxWords] = {0ull, 0ull};
    for (int w = 0; w < W; ++w) row[w] = (a < dx) ? rel[offA[c] + int64_t(a) * W + w] : 0ull;
    u32* out = reinterpret_cast<u32*>(rel + offB[c]);
    for (int bb = 0; bb < dy; bb += 32) {
      u32 mine = 0;
      for (int j = 0; j < 32; ++j) {
        const int b = bb + j;
        const u64 word = (b >> 6) ? row[1] : row[0];
        const u32 m = __ballot_sync(0xffffffffu, b < dy && ((word >> (b & 63)) & 1ull));
        if (lane == j) mine = m;
      }
      const int b = bb + lane;
      if (b < dy) out[(int64_t(b) * W) * 2 + g] = mine;
    }
  }
}

__global__ void k_static_finish(const unsigned char* scratch, StaticLayout L, int64_t* status) {
  const KStats* st = reinterpret_cast<const KStats*>(scratch + L.stats);
  status[0] = st->error ? 1 : st->inconsistent;
  status[1] = static_cast<int64_t>(st->deletions);
  status[2] = st->rounds_max;
  status[3] = st->error;
}

std::mutex g_static_mu;
void* g_static_ptr[128];
unsigned long long g_static_ctx[128];  // id of the context the address belongs to

// Unique id of the calling thread's current context (0 if none, or if the
// driver is too old to say), through driver entry points fetched by the
// runtime (the library does not link the driver library itself).
unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", reinterpret_cast<void**>(&get_current), 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      get_current = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", reinterpret_cast<void**>(&get_id), 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      get_id = nullptr;
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the static array on the current device, looked up with
// that device current on the first call and again whenever the device's
// current context has changed since.
int static_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return CP_E_CUDA;
  }
  if (dev < 0 || dev >= 128) {
    set_last_error("device index out of range");
    return CP_E_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_static_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_static_ptr[dev] || (ctx && ctx != g_static_ctx[dev])) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) {
      set_last_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return CP_E_CUDA;
    }
    g_static_ptr[dev] = p;
    // The lookup makes the device's primary context current if none was.
    g_static_ctx[dev] = ctx ? ctx : current_context_id();
  }
  *out = static_cast<unsigned char*>(g_static_ptr[dev]);
  return CP_OK;
}

}  // namespace
}  // namespace cpgpu

using namespace cpgpu;

extern "C" int cp_enforce_ac_static(int n, int W, const int* d_dom_size, uint64_t* d_dom, int n_bin,
                                    const int* d_bin_scope, const uint64_t* d_bin_rows, int64_t* d_status,
                                    void* stream) {
  if (n < 1 || n > kStaticMaxVars || W < 1 || W > kStaticMaxWords || n_bin < 0 || n_bin > kStaticMaxBin) {
    set_last_error("cp_enforce_ac_static: sizes beyond the limits (n <= 2048, W <= 2, n_bin <= 2048): n=" +
                     std::to_string(n) + " W=" + std::to_string(W) + " n_bin=" + std::to_string(n_bin));
    return CP_E_ARG;
  }
  if (!d_dom_size || !d_dom || !d_status || (n_bin > 0 && (!d_bin_scope || !d_bin_rows))) {
    set_last_error("cp_enforce_ac_static: null pointer argument");
    return CP_E_ARG;
  }
  unsigned char* scratch = nullptr;
  int rc = static_scratch(&scratch);
  if (rc != CP_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  DevNet N;
  N.n = n;
  N.W = W;
  N.nb = n_bin;
  N.nt = 0;
  N.chunk = kStaticChunk;
  N.total_values = int64_t(n) * 64 * W;
  const size_t cta_bytes = cta_state_bytes(N);
  const StaticLayout L = static_layout(n, W, n_bin, cta_bytes);
  if (L.total > kStaticScratchBytes) {
    set_last_error("cp_enforce_ac_static: network needs " + std::to_string(L.total) +
                     " bytes of scratch, more than the static " + std::to_string(kStaticScratchBytes));
    return CP_E_ARG;
  }
  N.dsize = d_dom_size;
  N.arc_start = reinterpret_cast<const int*>(scratch + L.arc_start);
  N.arcs = reinterpret_cast<const Arc*>(scratch + L.arcs);
  N.tinc_start = reinterpret_cast<const int*>(scratch + L.tinc);
  N.vtab = nullptr;
  N.rel = reinterpret_cast<const u64*>(scratch + L.rel);

  k_static_prep<<<1, 1024, 0, s>>>(n, W, n_bin, d_dom_size, d_bin_scope, reinterpret_cast<const u64*>(d_bin_rows),
                                   reinterpret_cast<u64*>(d_dom), scratch, L);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = launch_node(N, reinterpret_cast<u64*>(d_dom), 0, 0, kOpRoot, 0, 0, nullptr, 0,
                    reinterpret_cast<KStats*>(scratch + L.stats), nullptr, 256, scratch + L.cta, s);
  if (e == cudaSuccess) {
    k_static_finish<<<1, 1, 0, s>>>(scratch, L, d_status);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    set_last_error(std::string("cp_enforce_ac_static: ") + cudaGetErrorString(e));
    return CP_E_CUDA;
  }
  return CP_OK;
}
