// Support counting of SAC tiles: the bitwise test beside a tensor-core
// formulation on the 5th-generation tensor cores (tcgen05, accumulators in
// tensor memory).
//
// A tile is (x, y, z) with constraints joining x-y and y-z. Its 128 branches
// are x = a (a < dom(x)); branch a's domain of y is D_a(y) = D(y) & R(x=a -> y)
// (round one of the singleton test of x = a). For every branch and every value
// v of z the question is whether v keeps a support in D_a(y): the AND-then-any
// of AC3bit::seek_support (src/AC3bit.cpp:29-38). As a matrix product it is
// C = A * B^T with A[a][c] = [c in D_a(y)] (M = 128 branches, K = 128 values of
// y) and B[v][c] = [(y = c, z = v) allowed] (N = 128 values of z): v loses every
// support in branch a iff C[a][v] = 0. The 0/1 operands are exact in bf16 and
// the counts (at most 128) exact in fp32, so both kernels give the same bits:
//   out[tile][a] = the values v in D(z) with C[a][v] = 0 (two u64 words),
//   zero for a >= dom(x).
// k_tiles_bitwise: one warp per tile, 2-word ANDs and ballots.
// k_tiles_tc: one CTA of 128 threads per tile; each thread expands one row of
// A and one of B from bits into bf16 in shared memory (K-major, 128-byte
// swizzle), one thread issues the eight 128x128x16 MMAs into tensor memory and
// commits them to an mbarrier, then every thread reads its row of C (its
// tensor-memory lane) and forms the removal bits. Domains of up to 128 values.
#include <algorithm>
#include <cstdint>

#include "cp_internal.h"

namespace cpgpu {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kTcThreads = 128;
constexpr uint32_t kBf16One = 0x3F80u;
constexpr int kTcOperandBytes = 2 * 128 * 128;  // one 128x128 bf16 operand
constexpr int kTcSmem = 2 * kTcOperandBytes + 1024;  // A, B, alignment slack
// Instruction descriptor of tcgen05.mma kind::f16: D fp32 (bits 4-5 = 1),
// A and B bf16 (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N = 128 (bits 17-22 = N >> 3), M = 128 (bits 24-28 = M >> 4).
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
constexpr long long kTcWaitNs = 2000000000ll;  // bounded mbarrier wait

__device__ __forceinline__ long long gtimer() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle (rows of 128
// bytes, 8-row atoms of 1024 bytes, atoms 1024 bytes apart), version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
  d |= static_cast<uint64_t>(1) << 16;            // leading byte offset (not used by swizzled K-major)
  d |= static_cast<uint64_t>(1024 >> 4) << 32;    // stride byte offset between 8-row atoms
  d |= static_cast<uint64_t>(1) << 46;            // descriptor version
  d |= static_cast<uint64_t>(2) << 61;            // 128-byte swizzle
  return d;
}

// Row r of a 128x128 bf16 operand from 128 bits (two words): K elements
// 64j .. 64j+63 (word j) go to the 128-byte row r of region j (16 KB each),
// 16-byte piece p stored at piece p ^ (r & 7) of the row.
__device__ __forceinline__ void put_row_bits(unsigned char* region0, int r, u64 w0, u64 w1) {
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const u64 w = j ? w1 : w0;
    unsigned char* row = region0 + j * 16384 + (r >> 3) * 1024 + (r & 7) * 128;
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      const u32 b = static_cast<u32>(w >> (8 * p)) & 0xFFu;
      uint4 v;
      v.x = ((b & 1u) ? kBf16One : 0u) | ((b & 2u) ? kBf16One << 16 : 0u);
      v.y = ((b & 4u) ? kBf16One : 0u) | ((b & 8u) ? kBf16One << 16 : 0u);
      v.z = ((b & 16u) ? kBf16One : 0u) | ((b & 32u) ? kBf16One << 16 : 0u);
      v.w = ((b & 64u) ? kBf16One : 0u) | ((b & 128u) ? kBf16One << 16 : 0u);
      *reinterpret_cast<uint4*>(row + ((p ^ (r & 7)) << 4)) = v;
    }
  }
}

template <int WT>
__device__ __forceinline__ void load2(const u64* p, u64& a, u64& b) {
  a = p[0];
  b = WT > 1 ? p[1] : 0ull;
}

template <int WT>
__global__ void __launch_bounds__(256) k_tiles_bitwise(const u64* rel, const u64* dom, const SacTile* tiles,
                                                       int ntiles, u64* out) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int t = gw; t < ntiles; t += nw) {
    const SacTile T = tiles[t];
    u64 y0, y1, z0, z1;
    load2<WT>(dom + static_cast<size_t>(T.y) * WT, y0, y1);
    load2<WT>(dom + static_cast<size_t>(T.z) * WT, z0, z1);
    // Lane l holds the rows (over y) of z's values l, l + 32, l + 64, l + 96.
    u64 rz[4][2];
    bool live[4];
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const int v = g * 32 + lane;
      live[g] = v < T.dz && (((g < 2 ? z0 : z1) >> ((g & 1) * 32 + lane)) & 1ull);
      if (v < T.dz) {
        load2<WT>(rel + T.zy + static_cast<size_t>(v) * WT, rz[g][0], rz[g][1]);
      } else {
        rz[g][0] = rz[g][1] = 0;
      }
    }
    for (int base = 0; base < 128; base += 32) {
      const int a = base + lane;
      u64 d0 = 0, d1 = 0;
      if (a < T.dx) {
        load2<WT>(rel + T.xy + static_cast<size_t>(a) * WT, d0, d1);
        d0 &= y0;
        d1 &= y1;
      }
      u64 m0 = 0, m1 = 0;
      for (int j = 0; j < 32; ++j) {
        const u64 b0 = __shfl_sync(kFull, d0, j), b1 = __shfl_sync(kFull, d1, j);
        u32 m[4];
#pragma unroll
        for (int g = 0; g < 4; ++g) m[g] = __ballot_sync(kFull, live[g] && ((rz[g][0] & b0) | (rz[g][1] & b1)) == 0);
        if (lane == j) {
          m0 = static_cast<u64>(m[0]) | (static_cast<u64>(m[1]) << 32);
          m1 = static_cast<u64>(m[2]) | (static_cast<u64>(m[3]) << 32);
        }
      }
      if (a >= T.dx) m0 = m1 = 0;
      u64* o = out + (static_cast<size_t>(t) * 128 + a) * 2;
      o[0] = m0;
      o[1] = m1;
    }
  }
}

template <int WT>
__global__ void __launch_bounds__(kTcThreads) k_tiles_tc(const u64* rel, const u64* dom, const SacTile* tiles,
                                                         int ntiles, u64* out, int* err) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long s_mbar;
  __shared__ uint32_t s_tmem;
  __shared__ int s_bad;
  // Operands on 1024-byte boundaries (the swizzle atoms).
  const uint32_t raw = smem_addr(smem_raw);
  unsigned char* A = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  unsigned char* B = A + kTcOperandBytes;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t mbar = smem_addr(&s_mbar);
  if (tid == 0) {
    s_bad = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&s_tmem)),
                 "r"(128)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = s_tmem;
  uint32_t phase = 0;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const SacTile T = tiles[t];
    // Row tid of A (branch a = tid) and of B (value v = tid of z).
    u64 y0, y1, a0 = 0, a1 = 0, b0 = 0, b1 = 0;
    load2<WT>(dom + static_cast<size_t>(T.y) * WT, y0, y1);
    if (tid < T.dx) {
      load2<WT>(rel + T.xy + static_cast<size_t>(tid) * WT, a0, a1);
      a0 &= y0;
      a1 &= y1;
    }
    if (tid < T.dz) load2<WT>(rel + T.zy + static_cast<size_t>(tid) * WT, b0, b1);
    put_row_bits(A, tid, a0, a1);
    put_row_bits(B, tid, b0, b1);
    // Generic-proxy stores made visible to the tensor core (async proxy).
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t abase = smem_addr(A), bbase = smem_addr(B);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const uint32_t off = (k >> 2) * 16384 + (k & 3) * 32;  // K = 16k: region k/4, 32 bytes per step
        const uint64_t ad = sw128_desc(abase + off), bd = sw128_desc(bbase + off);
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(k)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                   : "memory");
    }
    // Every thread waits for the products (bounded by %globaltimer).
    {
      const long long t0 = gtimer();
      uint32_t done = 0;
      while (!done) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
        if (!done && gtimer() - t0 > kTcWaitNs) break;
      }
      if (!done) s_bad = 1;
    }
    phase ^= 1u;
    __syncthreads();
    if (s_bad) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // Row tid of C: tensor-memory lane tid (warp w reads lanes 32w..32w+31).
    u64 m0 = 0, m1 = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t c[32];
      const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + q * 32;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(c[0]), "=r"(c[1]), "=r"(c[2]), "=r"(c[3]), "=r"(c[4]), "=r"(c[5]), "=r"(c[6]), "=r"(c[7]),
            "=r"(c[8]), "=r"(c[9]), "=r"(c[10]), "=r"(c[11]), "=r"(c[12]), "=r"(c[13]), "=r"(c[14]), "=r"(c[15]),
            "=r"(c[16]), "=r"(c[17]), "=r"(c[18]), "=r"(c[19]), "=r"(c[20]), "=r"(c[21]), "=r"(c[22]),
            "=r"(c[23]), "=r"(c[24]), "=r"(c[25]), "=r"(c[26]), "=r"(c[27]), "=r"(c[28]), "=r"(c[29]),
            "=r"(c[30]), "=r"(c[31])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      u32 zero = 0;
#pragma unroll
      for (int i = 0; i < 32; ++i) zero |= (c[i] == 0u ? 1u : 0u) << i;
      if (q == 0) m0 |= zero;
      if (q == 1) m0 |= static_cast<u64>(zero) << 32;
      if (q == 2) m1 |= zero;
      if (q == 3) m1 |= static_cast<u64>(zero) << 32;
    }
    u64 z0, z1;
    load2<WT>(dom + static_cast<size_t>(T.z) * WT, z0, z1);
    const u64 lim0 = T.dz >= 64 ? ~0ull : ((1ull << T.dz) - 1ull);
    const u64 lim1 = T.dz >= 128 ? ~0ull : (T.dz <= 64 ? 0ull : ((1ull << (T.dz - 64)) - 1ull));
    m0 &= z0 & lim0;
    m1 &= z1 & lim1;
    if (tid >= T.dx) m0 = m1 = 0;
    u64* o = out + (static_cast<size_t>(t) * 128 + tid) * 2;
    o[0] = m0;
    o[1] = m1;
    // The next tile's products overwrite tensor memory after every read.
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  if (s_bad) {
    // A product that did not complete in time: give it one more bounded wait
    // before the tensor memory it writes is freed.
    if (tid == 0) {
      atomicExch(err, 1);
      const long long t0 = gtimer();
      uint32_t done = 0;
      while (!done && gtimer() - t0 < kTcWaitNs) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase ^ 1u)
            : "memory");
      }
    }
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128) : "memory");
}

}  // namespace

cudaError_t launch_tiles_bitwise(int W, const u64* rel, const u64* dom, const SacTile* tiles, int ntiles, u64* out,
                                 int sm_count, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  const int blocks = std::max(1, std::min((ntiles + 7) / 8, sm_count * 8));
  if (W == 1)
    k_tiles_bitwise<1><<<blocks, 256, 0, s>>>(rel, dom, tiles, ntiles, out);
  else if (W == 2)
    k_tiles_bitwise<2><<<blocks, 256, 0, s>>>(rel, dom, tiles, ntiles, out);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_tiles_tc(int W, const u64* rel, const u64* dom, const SacTile* tiles, int ntiles, u64* out,
                            int* err, int sm_count, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  if (W != 1 && W != 2) return cudaErrorInvalidValue;
  auto kern = W == 1 ? k_tiles_tc<1> : k_tiles_tc<2>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  // All of the unified L1 as shared memory, so that three CTAs fit per SM
  // from the first launch on.
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTcThreads, kTcSmem);
  if (e != cudaSuccess) return e;
  // At most four CTAs per SM: each holds 128 of the 512 tensor-memory columns.
  per_sm = std::max(1, std::min(per_sm, 4));
  const int blocks = std::max(1, std::min(ntiles, per_sm * sm_count));
  kern<<<blocks, kTcThreads, kTcSmem, s>>>(rel, dom, tiles, ntiles, out, err);
  return cudaGetLastError();
}

}  // namespace cpgpu
