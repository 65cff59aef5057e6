// Bitset-domain propagation kernels for sm_103a.
//
// One fixpoint body serves three launch shapes:
//   - k_node:  one CTA owns one network state (domains copied from a level
//              into shared memory); MAC nodes, small root ACs, and the plain
//              one-test-per-launch singleton baseline;
//   - k_sac:   persistent CTAs pull SAC singleton branches (x, a) from a
//              device work list; each branch gets its own domain copy in the
//              CTA's shared memory, only a 1-byte verdict leaves the SM;
//   - k_ac_front: the whole grid runs one fixpoint on global-memory domains
//              under a bounded grid barrier (cooperative launch), the
//              frontier kept as bitmaps instead of a queue.
//
// Frontier of the CTA-local fixpoints: a queue of the changed variables plus
// a bitmap that admits each once per round; a round's work items are the
// chunks of the queued variables' incidences, numbered by a CTA-wide scan.
// Round r processes queue r&1 and appends to the other; a variable's bit in
// the current bitmap is cleared by the warp that takes its first chunk, so
// both bitmaps are clean at every round boundary without a clearing pass.
//
// Revise of arc (z <- y) by one warp (the AND-then-any of AC3bit::seek_support,
// src/AC3bit.cpp:29-38, over all values of z at once): the warp either tests
// every live z value's support row against D(y) (32 values per ballot), or
// ORs the support rows of the live y values and intersects; it picks the side
// with fewer live values, so an assigned (singleton) y costs one row.
#include <algorithm>
#include <cstdio>
#include <type_traits>

#include "cp_gen.h"
#include "cp_internal.h"

namespace cpgpu {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ u64 vload(const u64* p) { return *reinterpret_cast<const volatile u64*>(p); }
__device__ __forceinline__ int vloadi(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

template <int WT>
__device__ __forceinline__ u64 sel(const u64 (&a)[WT], int i) {
  u64 v = 0;
#pragma unroll
  for (int w = 0; w < WT; ++w)
    if (w == i) v = a[w];
  return v;
}

template <int WT>
__device__ __forceinline__ void or_at(u64 (&a)[WT], int i, u64 m) {
#pragma unroll
  for (int w = 0; w < WT; ++w)
    if (w == i) a[w] |= m;
}

__device__ __forceinline__ u64 warp_or64(u64 x) {
  const u32 lo = __reduce_or_sync(kFull, static_cast<u32>(x));
  const u32 hi = __reduce_or_sync(kFull, static_cast<u32>(x >> 32));
  return (static_cast<u64>(hi) << 32) | lo;
}

__device__ __forceinline__ u64 shfl64(u64 x, int src) {
  const u32 lo = __shfl_sync(kFull, static_cast<u32>(x), src);
  const u32 hi = __shfl_sync(kFull, static_cast<u32>(x >> 32), src);
  return (static_cast<u64>(hi) << 32) | lo;
}

// A domain of WT words from shared memory, 128 bits per load (16-byte aligned for WT >= 2).
template <int WT>
__device__ __forceinline__ void load_sh(const u64* p, u64 (&r)[WT]) {
  if constexpr (WT == 1) {
    r[0] = p[0];
  } else {
#pragma unroll
    for (int h = 0; h < WT / 2; ++h) {
      const ulonglong2 v = reinterpret_cast<const ulonglong2*>(p)[h];
      r[2 * h] = v.x;
      r[2 * h + 1] = v.y;
    }
  }
}

// Support rows are read-only during a launch: non-coherent 128-bit loads.
template <int WT>
__device__ __forceinline__ void load_row(const u64* rel, size_t off, u64 (&r)[WT]) {
  if constexpr (WT == 1) {
    r[0] = __ldg(rel + off);
  } else {
    const ulonglong2* p = reinterpret_cast<const ulonglong2*>(rel + off);
#pragma unroll
    for (int h = 0; h < WT / 2; ++h) {
      const ulonglong2 v = __ldg(p + h);
      r[2 * h] = v.x;
      r[2 * h + 1] = v.y;
    }
  }
}

// Programmatic dependent launch: a kernel started by launch_pdl may be
// scheduled while the previous kernel of its stream is still finishing; it
// waits here, before its first memory access, for that kernel to complete
// and its writes to be visible. Without the launch attribute this is a no-op.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ long long globaltimer_ns() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// State of one fixpoint; pointers are shared or global memory.
struct Fix {
  u64* D;
  u32* q0;       // queued variables of the even / odd rounds (n each)
  u32* q1;
  int* pre;      // [n+1] first work item of each queued variable this round
  u32* fb0;
  u32* fb1;
  int* qlen;     // [3]
  int* tstamp;   // [nt] or null
  int* failed;   // [2] per round parity
  int* fail_var;
  int stamp_base;
};

struct Cnt {
  u64 rev = 0, rows = 0, tuples = 0, dels = 0;
};

// Domains and flags are shrunk concurrently by other warps, so lanes of one
// warp reading them separately may see different snapshots. Every value that
// steers warp-collective code (ballot, reduce, shuffle) is therefore read once
// and made warp-uniform: a domain is loaded one word per lane and broadcast;
// flags go through __any_sync. Call only from warp-converged code.
template <int WT>
__device__ __forceinline__ void load_dom_uniform(const u64* p, u64 (&d)[WT]) {
  const int lane = threadIdx.x & 31;
  const u64 mine = (lane < WT) ? vload(p + lane) : 0ull;
#pragma unroll
  for (int w = 0; w < WT; ++w) d[w] = __shfl_sync(kFull, mine, w);
}

__device__ __forceinline__ bool any_failed(const Fix& F) {
  return __any_sync(kFull, (vloadi(F.failed) | vloadi(F.failed + 1)) != 0);
}

__device__ __forceinline__ void set_failed(const Fix& F, int slot, int var) {
  atomicExch(F.failed + slot, 1);
  if (F.fail_var) atomicExch(F.fail_var, var);
}

__device__ __forceinline__ int incidences(const DevNet& N, int z) {
  return (N.arc_start[z + 1] - N.arc_start[z]) + (N.tinc_start[z + 1] - N.tinc_start[z]);
}

// Work items of variable z: its incidences in chunks of N.chunk (at least one).
__device__ __forceinline__ int var_chunks(const DevNet& N, int z) {
  return max(1, (incidences(N, z) + N.chunk - 1) / N.chunk);
}

// Admits z to the next round once (bitmap): one queue entry per variable.
__device__ __forceinline__ void append_var(u32* q, u32* fb, int* qlen, int z) {
  const u32 bit = 1u << (z & 31);
  const u32 old = atomicOr(fb + (z >> 5), bit);
  if (old & bit) return;
  q[atomicAdd(qlen, 1)] = static_cast<u32>(z);
}

// Seeds variable z (single thread): a seeded variable with an empty domain is
// a wipe-out.
template <int WT>
__device__ __forceinline__ void seed_var(const DevNet& N, const Fix& F, int z) {
  u64 any = 0;
#pragma unroll
  for (int w = 0; w < WT; ++w) any |= vload(F.D + static_cast<size_t>(z) * WT + w);
  if (!any) {
    set_failed(F, 0, z);
    return;
  }
  append_var(F.q0, F.fb0, F.qlen, z);
}

// Removes rm (warp-uniform) from D(z); on a change, checks for wipe-out and
// admits z to the next round.
template <int WT>
__device__ __forceinline__ void commit(const DevNet& N, const Fix& F, u32* qn, u32* fbn, int* qlenn, int slot, int z,
                                       const u64 (&rm)[WT], Cnt& cn) {
  const int lane = threadIdx.x & 31;
  bool any = false;
#pragma unroll
  for (int w = 0; w < WT; ++w) any |= rm[w] != 0;
  if (!any) return;
  u64 newly = 0;
  if (lane < WT) {
    const u64 r = sel<WT>(rm, lane);
    if (r) {
      const u64 old = atomicAnd(F.D + static_cast<size_t>(z) * WT + lane, ~r);
      newly = old & r;
    }
  }
  if (__ballot_sync(kFull, newly != 0) == 0) return;
  cn.dels += __popcll(newly);
  __threadfence_block();
  const u64 cur = (lane < WT) ? vload(F.D + static_cast<size_t>(z) * WT + lane) : 0ull;
  const bool nonempty = __ballot_sync(kFull, cur != 0) != 0;
  if (lane == 0) {
    if (!nonempty)
      set_failed(F, slot, z);
    else
      append_var(qn, fbn, qlenn, z);
  }
}

// Values of D(z) without a support in D(y) along arc A (dy, dz warp-uniform),
// from the union of the supports (in z) of the live values of y, 32 rows per
// step; stops as soon as the union covers D(z) (nothing to remove). The side
// to take when y has fewer live values than z.
template <int WT>
__device__ __forceinline__ void union_removals(const DevNet& N, const Arc A, const u64 (&dy)[WT], const u64 (&dz)[WT],
                                               u64 (&rm)[WT], Cnt& cn) {
  const int lane = threadIdx.x & 31;
  u64 acc[WT], cov[WT];
#pragma unroll
  for (int w = 0; w < WT; ++w) acc[w] = cov[w] = 0;
  int loaded = 0;
  bool covered = false;
#pragma unroll
  for (int base = 0; base < 64 * WT; base += 32) {
    if (covered) break;
    const u32 bits = static_cast<u32>(dy[base >> 6] >> (base & 32));
    if (bits == 0) continue;
    if ((bits >> lane) & 1u) {
      u64 r[WT];
      load_row<WT>(N.rel, A.yz + static_cast<size_t>(base + lane) * WT, r);
#pragma unroll
      for (int w = 0; w < WT; ++w) acc[w] |= r[w];
    }
    loaded += __popc(bits);
    u64 gap = 0;
#pragma unroll
    for (int w = 0; w < WT; ++w) {
      cov[w] = warp_or64(acc[w]);
      gap |= dz[w] & ~cov[w];
    }
    covered = gap == 0;
  }
#pragma unroll
  for (int w = 0; w < WT; ++w) rm[w] = dz[w] & ~cov[w];
  if (lane == 0) cn.rows += loaded;
}

// Value-wise removals: every live value of z tests its support row against
// D(y), one group of 32 values at a time.
template <int WT>
__device__ __forceinline__ void valuewise_removals_seq(const DevNet& N, u32 zy, const u64 (&dy)[WT],
                                                       const u64 (&dz)[WT], u64 (&rm)[WT]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int base = 0; base < 64 * WT; base += 32) {
    const u32 bits = static_cast<u32>(dz[base >> 6] >> (base & 32));
    if (bits == 0) continue;
    bool unsup = false;
    if ((bits >> lane) & 1u) {
      u64 r[WT];
      load_row<WT>(N.rel, zy + static_cast<size_t>(base + lane) * WT, r);
      u64 hit = 0;
#pragma unroll
      for (int w = 0; w < WT; ++w) hit |= r[w] & dy[w];
      unsup = hit == 0;
    }
    const u32 m = __ballot_sync(kFull, unsup);
    rm[base >> 6] |= static_cast<u64>(m) << (base & 32);
  }
}

// Revises z against y along arc A; dy / cy: D(y) and its size.
template <int WT>
__device__ __forceinline__ void revise_arc(const DevNet& N, const Fix& F, u32* qn, u32* fbn, int* qlenn, int slot,
                                           int y, const u64 (&dy)[WT], int cy, const Arc A, Cnt& cn) {
  const int lane = threadIdx.x & 31;
  const int z = A.z;
  u64 dz[WT];
  load_dom_uniform<WT>(F.D + static_cast<size_t>(z) * WT, dz);
  int cz = 0;
#pragma unroll
  for (int w = 0; w < WT; ++w) cz += __popcll(dz[w]);
  if (lane == 0) ++cn.rev;
  if (cy == 0 || cz == 0) {
    if (lane == 0) set_failed(F, slot, cy == 0 ? y : z);
    return;
  }
  u64 rm[WT];
#pragma unroll
  for (int w = 0; w < WT; ++w) rm[w] = 0;
  if (cy < cz) {
    union_removals<WT>(N, A, dy, dz, rm, cn);
  } else {
    valuewise_removals_seq<WT>(N, A.zy, dy, dz, rm);
    if (lane == 0) cn.rows += cz;
  }
  commit<WT>(N, F, qn, fbn, qlenn, slot, z, rm, cn);
}

// OR over the lanes of gmask (group-uniform result).
__device__ __forceinline__ u64 group_or64(u64 x, u32 gmask) {
  const u32 lo = __reduce_or_sync(gmask, static_cast<u32>(x));
  const u32 hi = __reduce_or_sync(gmask, static_cast<u32>(x >> 32));
  return (static_cast<u64>(hi) << 32) | lo;
}

// Revises na (2 .. 32 / G) arcs of y at once, arc g by the G lanes of group
// g (G = arc_group_lanes(WT)), with the same choice per arc as revise_arc:
// the union of the supports of D(y) when y has fewer live values than z, else
// each live value of z tests its row against D(y); G values per pass, one per
// lane. D(y) is warp-uniform, D(z) and everything that steers a group's
// collective calls group-uniform; groups without an arc stay idle.
template <int WT>
__device__ __forceinline__ void revise_arcs_grouped(const DevNet& N, const Fix& F, u32* qn, u32* fbn, int* qlenn,
                                                    int slot, int y, const Arc* arcs, int na, Cnt& cn) {
  constexpr int G = arc_group_lanes(WT);
  static_assert(G < 32, "grouped revision needs several arcs per warp");
  constexpr u32 kLow = (1u << G) - 1u;
  const int lane = threadIdx.x & 31, g = lane / G, li = lane % G;
  const u32 gmask = kLow << (g * G);
  const bool act = g < na;
  const Arc A = arcs[act ? g : 0];
  const int z = A.z;
  u64 dy[WT];
  load_dom_uniform<WT>(F.D + static_cast<size_t>(y) * WT, dy);
  const u64 mine = li < WT ? vload(F.D + static_cast<size_t>(z) * WT + li) : 0ull;
  u64 dz[WT];
  int cy = 0, cz = 0;
#pragma unroll
  for (int w = 0; w < WT; ++w) {
    dz[w] = __shfl_sync(kFull, mine, w, G);
    cy += __popcll(dy[w]);
    cz += __popcll(dz[w]);
  }
  if (act && li == 0) ++cn.rev;
  const bool empty = cy == 0 || cz == 0;
  if (act && empty && li == 0) set_failed(F, slot, cy == 0 ? y : z);
  const bool live = act && !empty;
  const bool by_union = cy < cz;
  const u32 off = by_union ? A.yz : A.zy;
  u64 acc[WT], rm[WT];
#pragma unroll
  for (int w = 0; w < WT; ++w) acc[w] = rm[w] = 0;
  bool done = !live;
#pragma unroll
  for (int base = 0; base < 64 * WT; base += G) {
    const u64 src = by_union ? dy[base >> 6] : dz[base >> 6];
    const u32 bits = done ? 0u : static_cast<u32>(src >> (base & 63)) & kLow;
    if (__ballot_sync(kFull, bits != 0) == 0) continue;
    bool unsup = false;
    if ((bits >> li) & 1u) {
      u64 r[WT];
      load_row<WT>(N.rel, off + static_cast<size_t>(base + li) * WT, r);
      ++cn.rows;
      u64 hit = 0;
#pragma unroll
      for (int w = 0; w < WT; ++w) {
        acc[w] |= r[w];
        hit |= r[w] & dy[w];
      }
      unsup = !by_union && hit == 0;
    }
    const u32 m = __ballot_sync(kFull, unsup);
    rm[base >> 6] |= static_cast<u64>((m >> (g * G)) & kLow) << (base & 63);
    if (by_union && !done) {
      u64 gap = 0;
#pragma unroll
      for (int w = 0; w < WT; ++w) gap |= dz[w] & ~group_or64(acc[w], gmask);
      done = gap == 0;
    }
  }
  if (by_union) {
#pragma unroll
    for (int w = 0; w < WT; ++w) rm[w] = dz[w] & ~group_or64(acc[w], gmask);
  }
  // Commit: remove rm from D(z); a group whose removal changed D(z) checks
  // for wipe-out and admits z to the next round.
  u64 newly = 0;
  if (live && li < WT) {
    const u64 r = sel<WT>(rm, li);
    if (r) {
      const u64 old = atomicAnd(F.D + static_cast<size_t>(z) * WT + li, ~r);
      newly = old & r;
    }
  }
  const u32 nb = __ballot_sync(kFull, newly != 0);
  if (nb == 0) return;
  cn.dels += __popcll(newly);
  __threadfence_block();
  const bool changed = (nb & gmask) != 0;
  const u64 cur = (changed && li < WT) ? vload(F.D + static_cast<size_t>(z) * WT + li) : 0ull;
  const u32 ne = __ballot_sync(kFull, cur != 0);
  if (changed && li == 0) {
    if ((ne & gmask) == 0)
      set_failed(F, slot, z);
    else
      append_var(qn, fbn, qlenn, z);
  }
}

// Table revision (GAC on a positive table, the definition of
// samples/verify_gac.cpp:121-164): a tuple is valid iff every coordinate is
// in its variable's domain; each scope variable keeps exactly the values that
// appear in a valid tuple. Lanes stride over tuples, projections are OR-reduced
// across the warp.
// Table t against the current domains D: rm[i] = the values of scope
// position i that appear in no valid tuple (s[i]: the scope, r: the arity).
// Returns a scope variable found empty (nothing computed then), or -1.
template <int WT>
__device__ __forceinline__ int table_removals(const DevNet& N, const u64* D, int t, int (&s)[kMaxArity], int& r,
                                              u64 (&rm)[kMaxArity][WT], Cnt& cn) {
  const int lane = threadIdx.x & 31;
  r = N.t_arity[t];
  u64 snap[kMaxArity][WT], proj[kMaxArity][WT];
  int empty_var = -1;
#pragma unroll
  for (int i = 0; i < kMaxArity; ++i) {
    s[i] = i < r ? N.t_scope4[t * kMaxArity + i] : 0;
    u64 any = 0;
    if (i < r) {
      load_dom_uniform<WT>(D + static_cast<size_t>(s[i]) * WT, snap[i]);
    } else {
#pragma unroll
      for (int w = 0; w < WT; ++w) snap[i][w] = 0;
    }
#pragma unroll
    for (int w = 0; w < WT; ++w) {
      proj[i][w] = 0;
      rm[i][w] = 0;
      any |= snap[i][w];
    }
    if (i < r && any == 0) empty_var = s[i];
  }
  if (lane == 0) ++cn.rev;
  if (empty_var >= 0) return empty_var;
  const int nt = N.t_ntup[t];
  const uint16_t* tp = N.t_tup + N.t_off[t];
  // Four tuples per lane per step, all coordinates loaded before any test.
  constexpr int kU = 4;
  for (int k0 = lane; k0 < nt; k0 += 32 * kU) {
    int v[kU][kMaxArity];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const int k = k0 + 32 * u;
#pragma unroll
      for (int i = 0; i < kMaxArity; ++i) v[u][i] = (i < r && k < nt) ? tp[static_cast<size_t>(i) * nt + k] : 0;
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      bool valid = k0 + 32 * u < nt;
#pragma unroll
      for (int i = 0; i < kMaxArity; ++i)
        if (i < r) valid = valid && ((sel<WT>(snap[i], v[u][i] >> 6) >> (v[u][i] & 63)) & 1ull);
      if (valid) {
#pragma unroll
        for (int i = 0; i < kMaxArity; ++i)
          if (i < r) or_at<WT>(proj[i], v[u][i] >> 6, 1ull << (v[u][i] & 63));
      }
    }
  }
  if (lane == 0) cn.tuples += nt;
#pragma unroll
  for (int i = 0; i < kMaxArity; ++i)
    if (i < r) {
#pragma unroll
      for (int w = 0; w < WT; ++w) rm[i][w] = snap[i][w] & ~warp_or64(proj[i][w]);
    }
  return -1;
}

// Tables the register path above does not take (arity above kMaxArity, or
// domains of more than 256 values): the scope positions are revised kG at a
// time. A group's domains are snapshot in registers and its projections built
// from the tuples valid against that snapshot and, at the other positions,
// against the domains in memory; the group's removals are committed
// (commit_fn(z, rm)) before the next group is computed. Domains only shrink,
// so a tuple found invalid against a later state is invalid in every later
// one and each removal is sound; a tuple counted valid on an earlier state of
// another scope variable is looked at again when that variable's change
// re-admits the table. Returns a scope variable found empty, or -1. Kept out
// of line: its registers would otherwise count against every fixpoint kernel
// that can meet a table.
template <int WT, int kG, class CommitFn>
__device__ __noinline__ int table_wide(const DevNet& N, const Fix& F, int t, Cnt& cn, CommitFn&& commit_fn) {
  const int lane = threadIdx.x & 31;
  const int r = N.t_arity[t];
  const int* sc = N.t_scope + N.t_soff[t];
  const int nt = N.t_ntup[t];
  const uint16_t* tp = N.t_tup + N.t_off[t];
  if (lane == 0) ++cn.rev;
  for (int g0 = 0; g0 < r; g0 += kG) {
    if (g0 > 0 && any_failed(F)) return -1;
    int s[kG];
    u64 snap[kG][WT], proj[kG][WT];
    int empty_var = -1;
#pragma unroll
    for (int i = 0; i < kG; ++i) {
      const bool in = g0 + i < r;
      s[i] = in ? sc[g0 + i] : 0;
      if (in) {
        load_dom_uniform<WT>(F.D + static_cast<size_t>(s[i]) * WT, snap[i]);
      } else {
#pragma unroll
        for (int w = 0; w < WT; ++w) snap[i][w] = 0;
      }
      u64 any = 0;
#pragma unroll
      for (int w = 0; w < WT; ++w) {
        proj[i][w] = 0;
        any |= snap[i][w];
      }
      if (in && any == 0) empty_var = s[i];
    }
    if (empty_var >= 0) return empty_var;
    for (int k = lane; k < nt; k += 32) {
      int v[kG];
      bool valid = true;
#pragma unroll
      for (int i = 0; i < kG; ++i) {
        v[i] = g0 + i < r ? tp[static_cast<size_t>(g0 + i) * nt + k] : 0;
        if (g0 + i < r) valid = valid && ((sel<WT>(snap[i], v[i] >> 6) >> (v[i] & 63)) & 1ull);
      }
      for (int j = 0; j < r && valid; ++j) {
        if (j >= g0 && j < g0 + kG) continue;
        const int u = tp[static_cast<size_t>(j) * nt + k];
        valid = (vload(F.D + static_cast<size_t>(__ldg(sc + j)) * WT + (u >> 6)) >> (u & 63)) & 1ull;
      }
      if (valid) {
#pragma unroll
        for (int i = 0; i < kG; ++i)
          if (g0 + i < r) or_at<WT>(proj[i], v[i] >> 6, 1ull << (v[i] & 63));
      }
    }
    if (lane == 0) cn.tuples += nt;
#pragma unroll
    for (int i = 0; i < kG; ++i)
      if (g0 + i < r) {
        u64 rm[WT];
#pragma unroll
        for (int w = 0; w < WT; ++w) rm[w] = snap[i][w] & ~warp_or64(proj[i][w]);
        commit_fn(s[i], rm);
      }
  }
  return -1;
}

// Positions a table of the given arity and domain width is revised in at a
// time by table_wide (the register path takes the rest).
template <int WT>
constexpr int kWideGroup = WT <= 4 ? kMaxArity : 1;

template <int WT>
__device__ __forceinline__ void revise_table(const DevNet& N, const Fix& F, u32* qn, u32* fbn, int* qlenn, int slot,
                                             int t, Cnt& cn) {
  const int lane = threadIdx.x & 31;
  if constexpr (WT <= 4) {
    if (N.t_arity[t] <= kMaxArity) {
      int s[kMaxArity], r = 0;
      u64 rm[kMaxArity][WT];
      const int empty_var = table_removals<WT>(N, F.D, t, s, r, rm, cn);
      if (empty_var >= 0) {
        if (lane == 0) set_failed(F, slot, empty_var);
        return;
      }
#pragma unroll
      for (int i = 0; i < kMaxArity; ++i)
        if (i < r) commit<WT>(N, F, qn, fbn, qlenn, slot, s[i], rm[i], cn);
      return;
    }
  }
  const int empty_var = table_wide<WT, kWideGroup<WT>>(
      N, F, t, cn, [&](int z, const u64 (&rm)[WT]) { commit<WT>(N, F, qn, fbn, qlenn, slot, z, rm, cn); });
  if (empty_var >= 0 && lane == 0) set_failed(F, slot, empty_var);
}

// Work item c (chunk of incidences) of variable y. kGroup: items with several
// arcs left are revised by lane groups (revise_arcs_grouped) -- for the
// latency-bound single-CTA fixpoints of searches; the throughput-bound SAC
// branch and batch kernels keep one arc per warp, and their registers.
template <int WT, bool kTab, bool kGroup = true>
__device__ __forceinline__ void process_item(const DevNet& N, const Fix& F, int y, int c, u32* fbc, u32* qn, u32* fbn,
                                             int* qlenn, int slot, int stamp, Cnt& cn) {
  const int lane = threadIdx.x & 31;
  if (c == 0 && lane == 0) atomicAnd(fbc + (y >> 5), ~(1u << (y & 31)));
  const int a0 = N.arc_start[y], da = N.arc_start[y + 1] - a0;
  const int t0 = N.tinc_start[y], dt = N.tinc_start[y + 1] - t0;
  const int lo = c * N.chunk;
  const int hi = min(lo + N.chunk, da + dt);
  for (int i = lo; i < hi;) {
    if (i < da) {
      if (any_failed(F)) return;
      const int left = min(hi, da) - i;
      bool grouped = false;
      if constexpr (kGroup && arc_group_lanes(WT) < 32) {
        if (left >= 2) {
          // Several arcs left in the item: one lane group per arc.
          const int na = min(32 / arc_group_lanes(WT), left);
          revise_arcs_grouped<WT>(N, F, qn, fbn, qlenn, slot, y, N.arcs + a0 + i, na, cn);
          i += na;
          grouped = true;
        }
      }
      if (!grouped) {
        const Arc A = N.arcs[a0 + i];
        u64 dy[WT];
        load_dom_uniform<WT>(F.D + static_cast<size_t>(y) * WT, dy);
        int cy = 0;
#pragma unroll
        for (int w = 0; w < WT; ++w) cy += __popcll(dy[w]);
        revise_arc<WT>(N, F, qn, fbn, qlenn, slot, y, dy, cy, A, cn);
        ++i;
      }
    } else if constexpr (kTab) {
      if (any_failed(F)) return;
      const int t = N.vtab[t0 + i - da];
      ++i;
      int prev = 0;
      if (lane == 0) prev = atomicMax(F.tstamp + t, stamp);
      prev = __shfl_sync(kFull, prev, 0);
      if (prev >= stamp) continue;
      revise_table<WT>(N, F, qn, fbn, qlenn, slot, t, cn);
    } else {
      break;
    }
  }
}

// The round's work items: pre[i] = work items of the queued variables before
// q[i] (a CTA-wide exclusive scan of their chunk counts), pre[len] = all of
// them. Every thread of the CTA calls it; ends with the CTA synchronised.
__device__ __forceinline__ int cta_round_items(const DevNet& N, const u32* q, int len, int* pre) {
  __shared__ int s_w[32];
  __shared__ int s_carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (len <= 32) {
    // One warp scans a short queue (the usual round of a search node): one
    // barrier instead of the block scan's five.
    if (warp == 0) {
      const int v = lane < len ? var_chunks(N, static_cast<int>(q[lane])) : 0;
      int x = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
      }
      if (lane < len) pre[lane] = x - v;
      if (lane == 31) pre[len] = x;
    }
    __syncthreads();
    return pre[len];
  }
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (int base = 0; base < len; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const int v = i < len ? var_chunks(N, static_cast<int>(q[i])) : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_w[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = lane < nw ? s_w[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, w, o);
        if (lane >= o) w += y;
      }
      s_w[lane] = w;
    }
    __syncthreads();
    const int carry = s_carry;
    if (i < len) pre[i] = carry + (warp ? s_w[warp - 1] : 0) + x - v;
    __syncthreads();
    if (threadIdx.x == 0) s_carry = carry + s_w[nw - 1];
    __syncthreads();
  }
  const int total = s_carry;
  if (threadIdx.x == 0) pre[len] = total;
  __syncthreads();
  return total;
}

// CTA-local fixpoint; the caller has seeded queue 0 and synchronised.
// Returns the number of rounds; sets *err on a round-count overrun.
template <int WT, bool kTab, bool kGroup = true>
__device__ int cta_fixpoint(const DevNet& N, const Fix& F, Cnt& cn, int* err) {
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const long long max_rounds = N.total_values + 2;
  int r = 0;
  for (;; ++r) {
    const int cur = r & 1;
    const int len = vloadi(F.qlen + r % 3);
    const int fl = vloadi(F.failed + cur);
    if (len == 0 || fl) break;
    if (r > max_rounds) {
      if (threadIdx.x == 0) atomicExch(err, -4);
      break;
    }
    if (threadIdx.x == 0) F.qlen[(r + 2) % 3] = 0;
    const u32* qc = cur ? F.q1 : F.q0;
    u32* qn = cur ? F.q0 : F.q1;
    u32* fbc = cur ? F.fb1 : F.fb0;
    u32* fbn = cur ? F.fb0 : F.fb1;
    int* qlenn = F.qlen + (r + 1) % 3;
    const int items = cta_round_items(N, qc, len, F.pre);
    // Warp w takes items w, w + W, ...; its cursor into the queue only moves
    // forward (pre is increasing).
    int i = 0;
    for (int j = warp; j < items; j += nwarps) {
      while (F.pre[i + 1] <= j) ++i;
      process_item<WT, kTab, kGroup>(N, F, static_cast<int>(qc[i]), j - F.pre[i], fbc, qn, fbn, qlenn, cur ^ 1,
                             F.stamp_base + r + 1, cn);
    }
    __syncthreads();
  }
  return r;
}

// Layout of the CTA-local state inside a byte buffer.
struct CtaLayout {
  size_t d, q0, q1, pre, fb0, fb1, ts, total;
};

__host__ __device__ inline CtaLayout cta_layout(const DevNet& N) {
  CtaLayout L;
  auto up = [](size_t x) { return (x + 15) & ~size_t(15); };
  const size_t nw = (static_cast<size_t>(N.n) + 31) / 32;
  L.d = 0;
  L.q0 = up(L.d + static_cast<size_t>(N.n) * N.W * 8);
  L.q1 = up(L.q0 + static_cast<size_t>(N.n) * 4);
  L.pre = up(L.q1 + static_cast<size_t>(N.n) * 4);
  L.fb0 = up(L.pre + (static_cast<size_t>(N.n) + 1) * 4);
  L.fb1 = up(L.fb0 + nw * 4);
  L.ts = up(L.fb1 + nw * 4);
  L.total = up(L.ts + static_cast<size_t>(N.nt) * 4);
  return L;
}

__device__ __forceinline__ Fix make_cta_fix(const DevNet& N, char* base, int* qlen, int* failed, int* fail_var) {
  const CtaLayout L = cta_layout(N);
  Fix F;
  F.D = reinterpret_cast<u64*>(base + L.d);
  F.q0 = reinterpret_cast<u32*>(base + L.q0);
  F.q1 = reinterpret_cast<u32*>(base + L.q1);
  F.pre = reinterpret_cast<int*>(base + L.pre);
  F.fb0 = reinterpret_cast<u32*>(base + L.fb0);
  F.fb1 = reinterpret_cast<u32*>(base + L.fb1);
  F.tstamp = N.nt ? reinterpret_cast<int*>(base + L.ts) : nullptr;
  F.qlen = qlen;
  F.failed = failed;
  F.fail_var = fail_var;
  F.stamp_base = 0;
  return F;
}

// Copies n*WT words with 16-byte vector accesses where possible.
__device__ __forceinline__ void block_copy(u64* dst, const u64* src, size_t words) {
  if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
    const size_t h = words / 2;
    const ulonglong2* s = reinterpret_cast<const ulonglong2*>(src);
    ulonglong2* d = reinterpret_cast<ulonglong2*>(dst);
    for (size_t i = threadIdx.x; i < h; i += blockDim.x) d[i] = s[i];
    if ((words & 1) && threadIdx.x == 0) dst[words - 1] = src[words - 1];
  } else {
    for (size_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  }
}

__device__ __forceinline__ void block_zero(u32* p, size_t n) {
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) p[i] = 0;
}

__device__ __forceinline__ void flush_counts(KStats* st, const Cnt& cn) {
  // Warp-reduce then one atomic per warp.
  u64 rev = cn.rev, rows = cn.rows, tuples = cn.tuples, dels = cn.dels;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    rev += __shfl_xor_sync(kFull, rev, o);
    rows += __shfl_xor_sync(kFull, rows, o);
    tuples += __shfl_xor_sync(kFull, tuples, o);
    dels += __shfl_xor_sync(kFull, dels, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (rev) atomicAdd(&st->revisions, rev);
    if (rows) atomicAdd(&st->rows, rows);
    if (tuples) atomicAdd(&st->tuples, tuples);
    if (dels) atomicAdd(&st->deletions, dels);
  }
}

// ---------------------------------------------------------------------------
// k_node: one CTA, one network state.
// ---------------------------------------------------------------------------
template <int WT, bool kTab>
__global__ void __launch_bounds__(512) k_node(DevNet N, u64* levels, int src, int dst, int op, int var, int val,
                                               const int* evt, int nevt, KStats* st, uint8_t* ok_out,
                                               char* gscratch) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_qlen[3], s_failed[2], s_failvar, s_err;
  char* base = gscratch ? gscratch : reinterpret_cast<char*>(smem_raw);
  Fix F = make_cta_fix(N, base, s_qlen, s_failed, &s_failvar);
  const size_t words = static_cast<size_t>(N.n) * WT;
  const CtaLayout L = cta_layout(N);
  block_copy(F.D, levels + static_cast<size_t>(src) * words, words);
  block_zero(reinterpret_cast<u32*>(base + L.fb0), (L.ts - L.fb0) / 4);
  if (N.nt) block_zero(reinterpret_cast<u32*>(F.tstamp), N.nt);
  if (threadIdx.x == 0) {
    s_qlen[0] = s_qlen[1] = s_qlen[2] = 0;
    s_failed[0] = s_failed[1] = 0;
    s_failvar = -1;
    s_err = 0;
  }
  __syncthreads();
  if (op == kOpRoot) {
    for (int z = threadIdx.x; z < N.n; z += blockDim.x) seed_var<WT>(N, F, z);
  } else if (op == kOpEvents) {
    for (int i = threadIdx.x; i < nevt; i += blockDim.x) seed_var<WT>(N, F, evt[i]);
  } else if (threadIdx.x == 0) {
    u64* dv = F.D + static_cast<size_t>(var) * WT;
    if (op == kOpAssign || op == kOpSingleton) {
      for (int w = 0; w < WT; ++w) dv[w] = (w == (val >> 6)) ? (1ull << (val & 63)) : 0ull;
    } else {  // refute
      dv[val >> 6] &= ~(1ull << (val & 63));
    }
    seed_var<WT>(N, F, var);
  }
  __syncthreads();
  Cnt cn;
  const int rounds = cta_fixpoint<WT, kTab>(N, F, cn, &s_err);
  const bool failed = (s_failed[0] | s_failed[1]) != 0;
  if (op != kOpSingleton) block_copy(levels + static_cast<size_t>(dst) * words, F.D, words);
  flush_counts(st, cn);
  if (threadIdx.x == 0) {
    st->inconsistent = failed ? 1 : 0;
    st->fail_var = s_failvar;
    atomicMax(&st->rounds_max, rounds);
    atomicAdd(&st->fixpoints, 1ull);
    if (s_err) st->error = s_err;
    if (ok_out) *ok_out = failed ? 0 : 1;
  }
}

// ---------------------------------------------------------------------------
// k_mac: the MAC search of MAC::enforce (src/MAC.cpp:100-165) run by one CTA,
// with the per-level "assigned" flags of IntVar (src/Network.cpp:112-118,
// 235-256) and AssignedStack (src/Solver.cpp:36-56, 114-116) that decide the
// dom/min variable order (src/MAC.cpp:357-368). The CTA's shared-memory
// domains always hold the current search level; levels live in a global
// stack. Persistent CTAs take jobs from a cursor.
// ---------------------------------------------------------------------------
struct MacShared {
  int qlen[3], failed[2], failvar, err, job, val, stop;
  unsigned long long wmin[32];
};

// One fixpoint on the CTA domains after op (root: every variable seeded;
// assign: D(var) := {val}; refute: val removed from D(var)). Returns true if
// consistent.
template <int WT, bool kTab>
__device__ bool mac_fix(const DevNet& N, const Fix& F, char* base, const CtaLayout& L, MacShared& sh, int op, int var,
                        int val, Cnt& cn) {
  block_zero(reinterpret_cast<u32*>(base + L.fb0), (L.ts - L.fb0) / 4);
  if (N.nt) block_zero(reinterpret_cast<u32*>(F.tstamp), N.nt);
  if (threadIdx.x == 0) {
    sh.qlen[0] = sh.qlen[1] = sh.qlen[2] = 0;
    sh.failed[0] = sh.failed[1] = 0;
  }
  __syncthreads();
  if (op == kOpRoot) {
    for (int z = threadIdx.x; z < N.n; z += blockDim.x) seed_var<WT>(N, F, z);
  } else if (threadIdx.x == 0) {
    u64* dv = F.D + static_cast<size_t>(var) * WT;
    if (op == kOpAssign) {
      for (int w = 0; w < WT; ++w) dv[w] = (w == (val >> 6)) ? (1ull << (val & 63)) : 0ull;
    } else {
      dv[val >> 6] &= ~(1ull << (val & 63));
    }
    seed_var<WT>(N, F, var);
  }
  __syncthreads();
  cta_fixpoint<WT, kTab>(N, F, cn, &sh.err);
  return (vloadi(&sh.failed[0]) | vloadi(&sh.failed[1])) == 0;
}

// First value of D(x) (VLH_MIN, src/MAC.cpp:338-340).
template <int WT>
__device__ __forceinline__ int dom_head(const u64* D, int x) {
#pragma unroll
  for (int w = 0; w < WT; ++w) {
    const u64 v = D[static_cast<size_t>(x) * WT + w];
    if (v) return w * 64 + __ffsll(static_cast<long long>(v)) - 1;
  }
  return -1;
}

// VRH_DOM_MIN: the first unassigned variable of strictly smaller domain size
// (smallest size, ties to the smallest index). Block-wide. With A_p null the
// candidates are the variables with more than one value instead
// (GModel::GetMinDomainVar, src/GModel.cu:1553-1572).
// With nbr (dom/deg, src/MAC.cpp:371-386) the key is |D(v)| / |neighbourhood(v)|
// in integers, -1 for a variable without neighbours; the first strict
// minimum in variable order either way (keys packed with the index).
template <int WT>
__device__ int mac_select(const u64* D, const uint8_t* A_p, int n, MacShared& sh, const int* nbr = nullptr) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  unsigned long long best = ~0ull;
  for (int v = threadIdx.x; v < n; v += blockDim.x) {
    if (A_p && A_p[v]) continue;
    int sz = 0;
#pragma unroll
    for (int w = 0; w < WT; ++w) sz += __popcll(D[static_cast<size_t>(v) * WT + w]);
    if (!A_p && sz <= 1) continue;
    // Keys offset by one so that dom/deg's -1 sorts first as an unsigned.
    const int k = nbr ? (nbr[v] == 0 ? -1 : sz / nbr[v]) : sz;
    const unsigned long long key = (static_cast<unsigned long long>(k + 1) << 32) | static_cast<unsigned>(v);
    best = key < best ? key : best;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long other = __shfl_xor_sync(kFull, best, o);
    best = other < best ? other : best;
  }
  if (lane == 0) sh.wmin[warp] = best;
  __syncthreads();
  if (warp == 0) {
    unsigned long long b = lane < nwarps ? sh.wmin[lane] : ~0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long other = __shfl_xor_sync(kFull, b, o);
      b = other < b ? other : b;
    }
    if (lane == 0) sh.wmin[0] = b;
  }
  __syncthreads();
  const unsigned long long b = sh.wmin[0];
  __syncthreads();
  return b == ~0ull ? -1 : static_cast<int>(b & 0xffffffffu);
}

// Runs job J for at most slice_ns of this launch (checked between nodes);
// a search still open then is suspended in J.state for the next launch.
template <int WT, bool kTab>
__device__ void mac_one(const DevNet& N, const MacJob& J, MacOut* out, char* base, MacShared& sh, long long slice_ns) {
  MacState& S = *J.state;
  if (S.phase == 2) return;
  Fix F = make_cta_fix(N, base, sh.qlen, sh.failed, &sh.failvar);
  const CtaLayout L = cta_layout(N);
  const int n = N.n;
  const size_t words = static_cast<size_t>(n) * WT;
  uint8_t* A = J.assigned;
  const long long t_enter = globaltimer_ns();
  if (threadIdx.x == 0) sh.err = 0;
  Cnt cn;
  long long npos = 0, nneg = 0, props = 0, t0 = t_enter;
  int status = -1, p = 0, top = 0;
  bool ok = true;
  if (S.phase == 0) {
    block_copy(F.D, J.init, words);
    for (size_t i = threadIdx.x; i < static_cast<size_t>(J.levels) * n; i += blockDim.x) A[i] = 0;
    __syncthreads();
    if (threadIdx.x == 0)
      for (int c = 0; c < J.n_choice; ++c) {
        const int2 ch = J.choices[c];
        u64* dv = F.D + static_cast<size_t>(ch.x) * WT;
        for (int w = 0; w < WT; ++w) dv[w] &= (w == (ch.y >> 6)) ? (1ull << (ch.y & 63)) : 0ull;
      }
    __syncthreads();
    props = 1;
    ok = mac_fix<WT, kTab>(N, F, base, L, sh, kOpRoot, 0, 0, cn);
    block_copy(J.stack_dom, F.D, words);
    if (!ok) status = 0;
  } else {
    p = S.p;
    top = S.top;
    npos = S.npos;
    nneg = S.nneg;
    props = S.props;
    t0 = S.t_start;
    block_copy(F.D, J.stack_dom + static_cast<size_t>(p) * words, words);
    __syncthreads();
  }
  bool suspended = false;
  while (status < 0) {
    if (threadIdx.x == 0) {
      const long long now = globaltimer_ns();
      sh.stop = (J.limit_ns > 0 && now - t0 > J.limit_ns) ? 1 : (slice_ns > 0 && now - t_enter > slice_ns ? 2 : 0);
    }
    __syncthreads();
    const int stop = sh.stop, err = sh.err;
    __syncthreads();
    if (err) {
      status = err;
      break;
    }
    if (stop == 1) {
      status = 2;
      break;
    }
    if (stop == 2) {
      suspended = true;
      break;
    }
    if (p + 1 >= J.levels) {
      status = -1;  // level stack too shallow
      break;
    }
    const int var = J.varh == 0 ? (p + 1 < n ? p + 1 : -1)
                                : mac_select<WT>(F.D, A + static_cast<size_t>(p) * n, n, sh, J.varh == 4 ? J.nbr : nullptr);
    if (var < 0) {
      status = -6;  // no variable to branch on
      break;
    }
    if (threadIdx.x == 0) sh.val = dom_head<WT>(F.D, var);
    // new_level(p): the flags of level p carry to level p + 1.
    for (int v = threadIdx.x; v < n; v += blockDim.x)
      A[static_cast<size_t>(p + 1) * n + v] = A[static_cast<size_t>(p) * n + v];
    top = p;
    __syncthreads();
    const int val = sh.val;
    if (threadIdx.x == 0) {
      J.path[p] = make_int2(var, val);
      A[static_cast<size_t>(p + 1) * n + var] = 1;
    }
    ++p;
    ++npos;
    ok = mac_fix<WT, kTab>(N, F, base, L, sh, kOpAssign, var, val, cn);
    ++props;
    block_copy(J.stack_dom + static_cast<size_t>(p) * words, F.D, words);
    if (ok && p == n) {
      for (int x = threadIdx.x; x < n; x += blockDim.x) J.solution[x] = dom_head<WT>(F.D, x);
      status = 1;
      break;
    }
    while (!ok && p > 0) {
      __syncthreads();
      const int2 va = J.path[p - 1];
      --p;
      // back_to(p): flags of levels p..top cleared.
      for (size_t i = static_cast<size_t>(p) * n + threadIdx.x; i < static_cast<size_t>(top + 1) * n; i += blockDim.x)
        A[i] = 0;
      top = p;
      ++nneg;
      block_copy(F.D, J.stack_dom + static_cast<size_t>(p) * words, words);
      ok = mac_fix<WT, kTab>(N, F, base, L, sh, kOpRefute, va.x, va.y, cn);
      ++props;
      block_copy(J.stack_dom + static_cast<size_t>(p) * words, F.D, words);
      // update_model_assigned: the decisions still on the path.
      for (int i = threadIdx.x; i < p; i += blockDim.x) A[static_cast<size_t>(p) * n + J.path[i].x] = 1;
      __syncthreads();
    }
    if (!ok) status = 0;
  }
  __syncthreads();
  if (suspended) {
    if (threadIdx.x == 0) {
      S.phase = 1;
      S.p = p;
      S.top = top;
      S.npos = npos;
      S.nneg = nneg;
      S.props = props;
      S.t_start = t0;
    }
    return;
  }
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0) {
    S.phase = 2;
    out->status = status;
    out->npos = npos;
    out->nneg = nneg;
    out->props = props;
    __threadfence_system();
    *reinterpret_cast<volatile int*>(&out->done) = 1;
  }
}

// First value of D(x) above a (VLH_MIN order; a = -1: the first value).
template <int WT>
__device__ __forceinline__ int dom_next(const u64* D, int x, int a) {
  const int from = a + 1;
#pragma unroll
  for (int w = 0; w < WT; ++w) {
    if ((w + 1) * 64 <= from) continue;
    u64 v = D[static_cast<size_t>(x) * WT + w];
    if (from > w * 64) v &= ~0ull << (from - w * 64);
    if (v) return w * 64 + __ffsll(static_cast<long long>(v)) - 1;
  }
  return -1;
}

// The d-way search of GModelSolver::Solve / Search (src/GModelSolver.cu:31-189)
// run by one CTA: at each level the smallest domain of more than one value,
// its values in increasing order, one fixpoint per child; a child that fails
// counts as a negative node. Level p's domains live in the global stack; the
// state a time slice leaves (depth, "entering level p") is resumed by the next
// launch, as for mac_one.
template <int WT, bool kTab>
__device__ void dway_one(const DevNet& N, const MacJob& J, MacOut* out, char* base, MacShared& sh,
                         long long slice_ns) {
  MacState& S = *J.state;
  if (S.phase == 2) return;
  Fix F = make_cta_fix(N, base, sh.qlen, sh.failed, &sh.failvar);
  const CtaLayout L = cta_layout(N);
  const int n = N.n;
  const size_t words = static_cast<size_t>(n) * WT;
  const long long t_enter = globaltimer_ns();
  if (threadIdx.x == 0) sh.err = 0;
  Cnt cn;
  long long npos = 0, nneg = 0, props = 0, t0 = t_enter;
  int status = -1, p = 0;
  bool fresh = true, dirty = false;
  if (S.phase == 0) {
    block_copy(F.D, J.init, words);
    __syncthreads();
    if (threadIdx.x == 0)
      for (int c = 0; c < J.n_choice; ++c) {
        const int2 ch = J.choices[c];
        u64* dv = F.D + static_cast<size_t>(ch.x) * WT;
        for (int w = 0; w < WT; ++w) dv[w] &= (w == (ch.y >> 6)) ? (1ull << (ch.y & 63)) : 0ull;
      }
    __syncthreads();
    props = 1;
    const bool ok = mac_fix<WT, kTab>(N, F, base, L, sh, kOpRoot, 0, 0, cn);
    block_copy(J.stack_dom, F.D, words);
    if (!ok) status = 0;
  } else {
    p = S.p;
    fresh = S.top != 0;
    npos = S.npos;
    nneg = S.nneg;
    props = S.props;
    t0 = S.t_start;
    dirty = true;
  }
  bool suspended = false;
  while (status < 0) {
    if (threadIdx.x == 0) {
      const long long now = globaltimer_ns();
      sh.stop = (fresh && J.limit_ns > 0 && now - t0 >= J.limit_ns) ? 1
                                                                     : (slice_ns > 0 && now - t_enter > slice_ns ? 2 : 0);
    }
    __syncthreads();
    const int stop = sh.stop, err = sh.err;
    __syncthreads();
    if (err) {
      status = err;
      break;
    }
    if (stop == 1) {
      status = 2;
      break;
    }
    if (stop == 2) {
      suspended = true;
      break;
    }
    if (dirty) {  // the CTA domains must hold level p
      block_copy(F.D, J.stack_dom + static_cast<size_t>(p) * words, words);
      __syncthreads();
      dirty = false;
    }
    if (fresh) {
      if (p + 1 >= J.levels) {
        status = -1;  // level stack too shallow
        break;
      }
      const int var = mac_select<WT>(F.D, nullptr, n, sh);
      if (var < 0) {  // every domain a singleton: a solution
        for (int x = threadIdx.x; x < n; x += blockDim.x) J.solution[x] = dom_head<WT>(F.D, x);
        status = 1;
        break;
      }
      if (threadIdx.x == 0) J.path[p] = make_int2(var, -1);
      fresh = false;
      __syncthreads();
    }
    const int2 pv = J.path[p];
    if (threadIdx.x == 0) sh.val = dom_next<WT>(F.D, pv.x, pv.y);
    __syncthreads();
    const int val = sh.val;
    __syncthreads();
    if (val < 0) {  // values of this level exhausted
      if (p == 0) {
        status = 0;
        break;
      }
      --p;
      dirty = true;
      continue;
    }
    if (threadIdx.x == 0) J.path[p].y = val;
    ++npos;
    const bool ok = mac_fix<WT, kTab>(N, F, base, L, sh, kOpAssign, pv.x, val, cn);
    ++props;
    if (!ok) {
      ++nneg;
      dirty = true;
      continue;
    }
    block_copy(J.stack_dom + static_cast<size_t>(p + 1) * words, F.D, words);
    ++p;
    fresh = true;
  }
  __syncthreads();
  if (suspended) {
    if (threadIdx.x == 0) {
      S.phase = 1;
      S.p = p;
      S.top = fresh ? 1 : 0;
      S.npos = npos;
      S.nneg = nneg;
      S.props = props;
      S.t_start = t0;
    }
    return;
  }
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0) {
    S.phase = 2;
    out->status = status;
    out->npos = npos;
    out->nneg = nneg;
    out->props = props;
    __threadfence_system();
    *reinterpret_cast<volatile int*>(&out->done) = 1;
  }
}

// A job runs the MAC search (varh 0 / 1) or the d-way search (varh 2).
template <int WT, bool kTab>
__device__ __forceinline__ void search_one(const DevNet& N, const MacJob& J, MacOut* out, char* base, MacShared& sh,
                                           long long slice_ns) {
  if (J.varh == 2)
    dway_one<WT, kTab>(N, J, out, base, sh, slice_ns);
  else
    mac_one<WT, kTab>(N, J, out, base, sh, slice_ns);
}

// Jobs of any domain width and network kind in one launch: each job runs the
// body instantiated for its width and table flag.
__global__ void __launch_bounds__(512) k_mac(const DevNet* nets, const MacJob* jobs, int njobs, int* cursor,
                                              MacOut* outs, char* gscratch, size_t gstride, long long slice_ns) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ MacShared sh;
  __shared__ DevNet sN;
  char* base = gscratch ? gscratch + blockIdx.x * gstride : reinterpret_cast<char*>(smem_raw);
  for (;;) {
    if (threadIdx.x == 0) {
      sh.job = atomicAdd(cursor, 1);
      if (sh.job < njobs) sN = nets[jobs[sh.job].net];
    }
    __syncthreads();
    const int j = sh.job;
    if (j >= njobs) break;
    const MacJob& J = jobs[j];
    MacOut* o = outs + j;
    const bool tab = sN.nt > 0;
    switch (sN.W) {
      case 1:
        tab ? search_one<1, true>(sN, J, o, base, sh, slice_ns) : search_one<1, false>(sN, J, o, base, sh, slice_ns);
        break;
      case 2:
        tab ? search_one<2, true>(sN, J, o, base, sh, slice_ns) : search_one<2, false>(sN, J, o, base, sh, slice_ns);
        break;
      case 4:
        tab ? search_one<4, true>(sN, J, o, base, sh, slice_ns) : search_one<4, false>(sN, J, o, base, sh, slice_ns);
        break;
      default:
        tab ? search_one<8, true>(sN, J, o, base, sh, slice_ns) : search_one<8, false>(sN, J, o, base, sh, slice_ns);
        break;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// k_sac: persistent CTAs over the SAC branch work list.
// ---------------------------------------------------------------------------
// gs_root (optional): a failed branch also removes its value from that
// level at once, so branches that start later in the sweep see it.
template <int WT, bool kTab>
__global__ void __launch_bounds__(256) k_sac(DevNet N, const u64* root, const int2* work, const int* nwork,
                                             int* cursor, uint8_t* ok, KStats* st, char* gscratch, size_t gstride,
                                             const int* idx, u64* gs_root) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_qlen[3], s_failed[2], s_failvar, s_err, s_b;
  char* base = gscratch ? gscratch + blockIdx.x * gstride : reinterpret_cast<char*>(smem_raw);
  Fix F = make_cta_fix(N, base, s_qlen, s_failed, &s_failvar);
  const CtaLayout L = cta_layout(N);
  const size_t words = static_cast<size_t>(N.n) * WT;
  const int total = *nwork;
  if (total == 0) return;  // an empty list (e.g. no deep branches): nothing to count either
  if (threadIdx.x == 0) s_err = 0;
  Cnt cn;
  int rounds_max = 0;
  u64 done = 0;
  for (;;) {
    if (threadIdx.x == 0) s_b = atomicAdd(cursor, 1);
    __syncthreads();
    const int i = s_b;
    if (i >= total) break;
    const int b = idx ? idx[i] : i;
    const int2 xa = work[b];
    block_copy(F.D, root, words);
    block_zero(reinterpret_cast<u32*>(base + L.fb0), (L.ts - L.fb0) / 4);
    if (N.nt) block_zero(reinterpret_cast<u32*>(F.tstamp), N.nt);
    if (threadIdx.x == 0) {
      s_qlen[0] = s_qlen[1] = s_qlen[2] = 0;
      s_failed[0] = s_failed[1] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      u64* dv = F.D + static_cast<size_t>(xa.x) * WT;
      for (int w = 0; w < WT; ++w) dv[w] = (w == (xa.y >> 6)) ? (1ull << (xa.y & 63)) : 0ull;
      append_var(F.q0, F.fb0, F.qlen, xa.x);
    }
    __syncthreads();
    const int rounds = cta_fixpoint<WT, kTab, false>(N, F, cn, &s_err);
    rounds_max = max(rounds_max, rounds);
    if (threadIdx.x == 0) {
      const bool failed = (s_failed[0] | s_failed[1]) != 0;
      ok[b] = failed ? 0 : 1;
      if (failed && gs_root) atomicAnd(gs_root + static_cast<size_t>(xa.x) * WT + (xa.y >> 6), ~(1ull << (xa.y & 63)));
    }
    ++done;
    __syncthreads();
  }
  flush_counts(st, cn);
  if (threadIdx.x == 0) {
    atomicMax(&st->rounds_max, rounds_max);
    if (done) {
      atomicAdd(&st->fixpoints, done);
      atomicAdd(&st->branches, done);
    }
    if (s_err) st->error = s_err;
  }
}

// ---------------------------------------------------------------------------
// Whole-grid fixpoints: a bounded grid barrier.
// ---------------------------------------------------------------------------
// Sense-free generation barrier; every block waits at most wait_ns, then
// reports CP_E_TIMEOUT through *err and returns false (a block that sees
// another's error stops waiting too, so every block leaves).
__device__ bool grid_barrier(unsigned* bar, unsigned nblocks, int* err, long long wait_ns) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned* vgen = bar + 1;
    const unsigned gen = *vgen;
    __threadfence();
    const unsigned arrived = atomicAdd(bar, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const long long t0 = globaltimer_ns();
      unsigned sleep = 32;
      while (*vgen == gen) {
        if (vloadi(err) != 0 || globaltimer_ns() - t0 > wait_ns) {
          atomicExch(err, -4);
          ok = 0;
          break;
        }
        __nanosleep(sleep);
        if (sleep < 1024) sleep <<= 1;
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---------------------------------------------------------------------------
// k_ac_front: the whole grid runs one fixpoint on global-memory domains, the
// frontier kept as bitmaps of changed variables (no work queue, no appends).
// Round r reads bitmap r%3 (the variables changed in round r-1), marks the
// variables it changes in bitmap (r+1)%3 and clears bitmap (r+2)%3, which
// round r+1 will write; flag[i] says that bitmap i has a bit set. A round's
// work is static: the binary incidences (arcs out of y, CSR by y) in groups
// of K, then the tables. A warp takes a group, tests the frontier bits of the
// group's source variables (one ballot: the active arcs, compacted by their
// rank in the ballot mask), reads D(y) and D(z) of all of them at once and
// then the support rows of all active arcs in one wave before testing any,
// so each warp keeps K revisions' loads in flight instead of one. A table is
// revised once per round when any of its scope variables changed. Warp w
// takes tasks w, w + W, ... and reads its next group's records while working
// on the current one. Failures of round r go to failed[(r+1)&1], which nobody
// writes during round r+1, so every block takes the same decision at the top
// of a round. Round 0 of a root fixpoint, where every variable is in the
// frontier, runs as a plain launch with one warp per task (k_front_first);
// the cooperative kernel then starts at round 1 and ends at once if round 0
// changed nothing.
// ---------------------------------------------------------------------------
template <int WT>
struct FrontGroup {
  static constexpr int K = WT == 1 ? 8 : (WT == 2 ? 4 : 1);
};
constexpr int kFrontBlock = 256;

__device__ __forceinline__ bool front_bit(const u32* bm, int v) { return (__ldcg(bm + (v >> 5)) >> (v & 31)) & 1u; }

// Removes rm (warp-uniform) from D(z); on a change, checks for wipe-out and
// marks z in the next frontier bitmap.
template <int WT>
__device__ __forceinline__ void commit_front(const Fix& F, u32* bn, int* fn, int slot, int z, const u64 (&rm)[WT],
                                             Cnt& cn) {
  const int lane = threadIdx.x & 31;
  bool any = false;
#pragma unroll
  for (int w = 0; w < WT; ++w) any |= rm[w] != 0;
  if (!any) return;
  bool emptied;
  if constexpr (WT == 1) {
    // One word: the atomic's old value says whether this removal emptied it.
    u64 old = 0;
    if (lane == 0) old = atomicAnd(F.D + z, ~rm[0]);
    old = shfl64(old, 0);
    const u64 newly = old & rm[0];
    if (!newly) return;
    if (lane == 0) cn.dels += __popcll(newly);
    emptied = (old & ~rm[0]) == 0;
  } else {
    u64 newly = 0;
    if (lane < WT) {
      const u64 r = sel<WT>(rm, lane);
      if (r) newly = atomicAnd(F.D + static_cast<size_t>(z) * WT + lane, ~r) & r;
    }
    if (__ballot_sync(kFull, newly != 0) == 0) return;
    cn.dels += __popcll(newly);
    __threadfence();
    const u64 cur = (lane < WT) ? vload(F.D + static_cast<size_t>(z) * WT + lane) : 0ull;
    emptied = __ballot_sync(kFull, cur != 0) == 0;
  }
  if (lane == 0) {
    if (emptied) {
      set_failed(F, slot, z);
    } else {
      const u32 bit = 1u << (z & 31);
      if (!(atomicOr(bn + (z >> 5), bit) & bit)) atomicExch(fn, 1);
    }
  }
}

// One group of up to K binary incidences: lane k < cnt holds incidence k's
// record A (read ahead by the caller). all: every variable is in the
// frontier (round 0 of a root fixpoint), no bitmap test (bc unused).
template <int WT>
__device__ __forceinline__ void front_group(const DevNet& N, const Fix& F, const Arc A, int cnt, bool all,
                                            const u32* bc, u32* bn, int* fn, int slot, Cnt& cn) {
  constexpr int K = FrontGroup<WT>::K;
  const int lane = threadIdx.x & 31;
  // D(y) and D(z) of each active incidence, lane k holding incidence k's.
  u64 dyL[WT], dzL[WT];
#pragma unroll
  for (int w = 0; w < WT; ++w) dyL[w] = dzL[w] = 0;
  const bool act = lane < cnt && (all || front_bit(bc, A.src));
  const u32 m = __ballot_sync(kFull, act);
  if (!m || any_failed(F)) return;
  if (act) {
#pragma unroll
    for (int w = 0; w < WT; ++w) {
      dyL[w] = vload(F.D + static_cast<size_t>(A.src) * WT + w);
      dzL[w] = vload(F.D + static_cast<size_t>(A.z) * WT + w);
    }
  }
  if constexpr (WT <= 2) {
    constexpr int kVG = 2 * WT;  // groups of 32 values of z
    u64 rows[K][kVG][WT];
    // The rows of z's live values of every active arc revised value-wise
    // (y has at least as many live values as z), all issued before any test.
#pragma unroll
    for (int k = 0; k < K; ++k) {
      u64 dz[WT];
      int cz = 0, cy = 0;
#pragma unroll
      for (int w = 0; w < WT; ++w) {
        dz[w] = shfl64(dzL[w], k);
        cz += __popcll(dz[w]);
        cy += __popcll(shfl64(dyL[w], k));
      }
      const u32 zy = __shfl_sync(kFull, A.zy, k);
      const bool vw = ((m >> k) & 1u) && cy >= cz && cz > 0;
#pragma unroll
      for (int g = 0; g < kVG; ++g) {
        const bool live = vw && ((dz[g >> 1] >> ((g & 1) * 32 + lane)) & 1ull);
        if (live) {
          load_row<WT>(N.rel, zy + static_cast<size_t>(g * 32 + lane) * WT, rows[k][g]);
        } else {
#pragma unroll
          for (int w = 0; w < WT; ++w) rows[k][g][w] = 0;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (!((m >> k) & 1u)) continue;
      u64 dz[WT], dy[WT], rm[WT];
      int cz = 0, cy = 0;
#pragma unroll
      for (int w = 0; w < WT; ++w) {
        dz[w] = shfl64(dzL[w], k);
        dy[w] = shfl64(dyL[w], k);
        cz += __popcll(dz[w]);
        cy += __popcll(dy[w]);
        rm[w] = 0;
      }
      const Arc Ak{__shfl_sync(kFull, A.z, k), __shfl_sync(kFull, A.zy, k), __shfl_sync(kFull, A.yz, k),
                   __shfl_sync(kFull, A.src, k)};
      if (lane == 0) ++cn.rev;
      if (cy == 0 || cz == 0) {
        if (lane == 0) set_failed(F, slot, cy == 0 ? Ak.src : Ak.z);
        return;
      }
      if (cy >= cz) {
#pragma unroll
        for (int g = 0; g < kVG; ++g) {
          const bool live = (dz[g >> 1] >> ((g & 1) * 32 + lane)) & 1ull;
          u64 hit = 0;
#pragma unroll
          for (int w = 0; w < WT; ++w) hit |= rows[k][g][w] & dy[w];
          const u32 um = __ballot_sync(kFull, live && hit == 0);
          rm[g >> 1] |= static_cast<u64>(um) << ((g & 1) * 32);
        }
        if (lane == 0) cn.rows += cz;
      } else {
        union_removals<WT>(N, Ak, dy, dz, rm, cn);
      }
      commit_front<WT>(F, bn, fn, slot, Ak.z, rm, cn);
    }
  } else {
    for (int k = 0; k < K; ++k) {
      if (!((m >> k) & 1u)) continue;
      u64 dz[WT], dy[WT], rm[WT];
      int cz = 0, cy = 0;
#pragma unroll
      for (int w = 0; w < WT; ++w) {
        dz[w] = shfl64(dzL[w], k);
        dy[w] = shfl64(dyL[w], k);
        cz += __popcll(dz[w]);
        cy += __popcll(dy[w]);
        rm[w] = 0;
      }
      const Arc Ak{__shfl_sync(kFull, A.z, k), __shfl_sync(kFull, A.zy, k), __shfl_sync(kFull, A.yz, k),
                   __shfl_sync(kFull, A.src, k)};
      if (lane == 0) ++cn.rev;
      if (cy == 0 || cz == 0) {
        if (lane == 0) set_failed(F, slot, cy == 0 ? Ak.src : Ak.z);
        return;
      }
      if (cy >= cz) {
        valuewise_removals_seq<WT>(N, Ak.zy, dy, dz, rm);
        if (lane == 0) cn.rows += cz;
      } else {
        union_removals<WT>(N, Ak, dy, dz, rm, cn);
      }
      commit_front<WT>(F, bn, fn, slot, Ak.z, rm, cn);
    }
  }
}

// Table t, if one of its scope variables is in the frontier.
template <int WT>
__device__ __forceinline__ void front_table(const DevNet& N, const Fix& F, int t, bool all, const u32* bc, u32* bn,
                                            int* fn, int slot, Cnt& cn) {
  const int lane = threadIdx.x & 31;
  const int ar = N.t_arity[t];
  bool act = false;
  if (ar <= kMaxArity) {
    act = lane < ar && (all || front_bit(bc, N.t_scope4[t * kMaxArity + lane]));
  } else {
    const int* sc = N.t_scope + N.t_soff[t];
    for (int p = lane; p < ar && !act; p += 32) act = all || front_bit(bc, sc[p]);
  }
  if (!__any_sync(kFull, act) || any_failed(F)) return;
  if constexpr (WT <= 4) {
    if (ar <= kMaxArity) {
      int s[kMaxArity], r = 0;
      u64 rm[kMaxArity][WT];
      const int empty_var = table_removals<WT>(N, F.D, t, s, r, rm, cn);
      if (empty_var >= 0) {
        if (lane == 0) set_failed(F, slot, empty_var);
        return;
      }
#pragma unroll
      for (int i = 0; i < kMaxArity; ++i)
        if (i < r) commit_front<WT>(F, bn, fn, slot, s[i], rm[i], cn);
      return;
    }
  }
  const int empty_var = table_wide<WT, kWideGroup<WT>>(
      N, F, t, cn, [&](int z, const u64 (&rm)[WT]) { commit_front<WT>(F, bn, fn, slot, z, rm, cn); });
  if (empty_var >= 0 && lane == 0) set_failed(F, slot, empty_var);
}

// Counters of the warps of one block summed in shared memory, then one global
// atomic per counter and block (every thread of the block must call it).
__device__ __forceinline__ void flush_counts_block(KStats* st, const Cnt& cn) {
  __shared__ unsigned long long s_c[4];
  if (threadIdx.x < 4) s_c[threadIdx.x] = 0;
  __syncthreads();
  u64 c[4] = {cn.rev, cn.rows, cn.tuples, cn.dels};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c[i] += __shfl_xor_sync(kFull, c[i], o);
    if ((threadIdx.x & 31) == 0 && c[i]) atomicAdd(&s_c[i], c[i]);
  }
  __syncthreads();
  // revisions, rows, tuples, deletions are consecutive fields of KStats.
  if (threadIdx.x < 4 && s_c[threadIdx.x]) atomicAdd(&st->revisions + threadIdx.x, s_c[threadIdx.x]);
}

__device__ __forceinline__ Fix make_front_fix(u64* D, const GridScratch& G, KStats* st) {
  Fix F;
  F.D = D;
  F.q0 = F.q1 = nullptr;
  F.pre = nullptr;
  F.fb0 = F.fb1 = nullptr;
  F.qlen = nullptr;
  F.tstamp = nullptr;
  F.failed = G.failed;
  F.fail_var = &st->fail_var;
  F.stamp_base = 0;
  return F;
}

// Round 0 of a root fixpoint: one warp per task, every variable in the
// frontier; changes go to bitmap 1 and flag 1, wipe-outs to failed[1] (an
// empty domain at the start too), where k_ac_front's round 1 reads them.
template <int WT, bool kTab>
__global__ void __launch_bounds__(kFrontBlock, WT <= 2 ? 2 : 1) k_front_first(DevNet N, u64* D, GridScratch G,
                                                                              KStats* st) {
  pdl_wait();
  const Fix F = make_front_fix(D, G, st);
  const int nw = (N.n + 31) >> 5;
  const int lane = threadIdx.x & 31;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gthreads = gridDim.x * blockDim.x;
  for (int z = gtid; z < N.n; z += gthreads) {
    u64 any = 0;
#pragma unroll
    for (int w = 0; w < WT; ++w) any |= vload(D + static_cast<size_t>(z) * WT + w);
    if (!any) set_failed(F, 1, z);
  }
  constexpr int K = FrontGroup<WT>::K;
  const int narcs = N.arc_start[N.n];
  const int ngroups = (narcs + K - 1) / K;
  const int task = gtid >> 5;
  Cnt cn;
  if (task < ngroups) {
    const int cnt = min(K, narcs - task * K);
    Arc a{0, 0, 0, 0};
    if (lane < cnt) a = N.arcs[task * K + lane];
    front_group<WT>(N, F, a, cnt, true, nullptr, G.bm + nw, G.flags + 1, 1, cn);
  } else if constexpr (kTab) {
    if (task < ngroups + N.nt) front_table<WT>(N, F, task - ngroups, true, nullptr, G.bm + nw, G.flags + 1, 1, cn);
  }
  flush_counts_block(st, cn);
  if (gtid == 0) atomicMax(&st->rounds_max, 1);
}

// Rounds from `first` on: first = 0 seeds the frontier with evt (the
// variables whose domains changed), first = 1 continues after k_front_first.
template <int WT, bool kTab>
__global__ void __launch_bounds__(kFrontBlock, WT <= 2 ? 2 : 1) k_ac_front(DevNet N, u64* D, const int* evt,
                                                                           const int* nevt_dev, int nevt, int first,
                                                                           GridScratch G, KStats* st) {
  const Fix F = make_front_fix(D, G, st);
  const int nw = (N.n + 31) >> 5;
  u32* B = G.bm;        // three bitmaps of nw words
  int* flag = G.flags;  // [3]
  const unsigned nblocks = gridDim.x;
  const int lane = threadIdx.x & 31;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gthreads = gridDim.x * blockDim.x;
  int* err = &st->grid_err;
  bool ok = true;
  if (first == 0) {
    const int ne = nevt_dev ? vloadi(nevt_dev) : nevt;
    for (int i = gtid; i < ne; i += gthreads) {
      const int z = evt[i];
      u64 any = 0;
#pragma unroll
      for (int w = 0; w < WT; ++w) any |= vload(D + static_cast<size_t>(z) * WT + w);
      if (!any) {
        set_failed(F, 0, z);
      } else {
        atomicOr(B + (z >> 5), 1u << (z & 31));
        atomicExch(flag, 1);
      }
    }
    ok = grid_barrier(G.bar, nblocks, err, G.wait_ns);
  }
  Cnt cn;
  const long long max_rounds = N.total_values + 2;
  constexpr int K = FrontGroup<WT>::K;
  const int narcs = N.arc_start[N.n];
  const int ngroups = (narcs + K - 1) / K;
  const int ntasks = ngroups + (kTab ? N.nt : 0);
  const int gwarp = gtid >> 5, nwarps = gthreads >> 5;
  int r = first;
  for (; ok; ++r) {
    const int cur = r % 3, nxt = (r + 1) % 3, clr = (r + 2) % 3;
    if (!vloadi(flag + cur) || vloadi(F.failed + (r & 1))) break;
    if (r > max_rounds) {
      if (gtid == 0) st->error = -4;
      break;
    }
    const u32* bc = B + static_cast<size_t>(cur) * nw;
    u32* bn = B + static_cast<size_t>(nxt) * nw;
    u32* bz = B + static_cast<size_t>(clr) * nw;
    for (int w = gtid; w < nw; w += gthreads) bz[w] = 0;
    if (gtid == 0) flag[clr] = 0;
    const int slot = (r + 1) & 1;
    Arc an{0, 0, 0, 0};
    if (gwarp < ngroups && lane < min(K, narcs - gwarp * K)) an = N.arcs[gwarp * K + lane];
    for (int t = gwarp; t < ntasks; t += nwarps) {
      const int tn = t + nwarps;
      if (t < ngroups) {
        const Arc a = an;
        if (tn < ngroups && lane < min(K, narcs - tn * K)) an = N.arcs[tn * K + lane];
        front_group<WT>(N, F, a, min(K, narcs - t * K), false, bc, bn, flag + nxt, slot, cn);
      } else if constexpr (kTab) {
        front_table<WT>(N, F, t - ngroups, false, bc, bn, flag + nxt, slot, cn);
      }
    }
    ok = grid_barrier(G.bar, nblocks, err, G.wait_ns);
  }
  flush_counts(st, cn);
  if (gtid == 0) {
    st->inconsistent = (vloadi(F.failed) | vloadi(F.failed + 1)) ? 1 : 0;
    atomicMax(&st->rounds_max, r);
    atomicAdd(&st->fixpoints, 1ull);
  }
}

// ---------------------------------------------------------------------------
// k_ac3_replay: AC3::enforce (src/AC3.cpp:99-141, with AC3bit's seek_support,
// src/AC3bit.cpp:29-38, and the FIFO var_que, src/Solver.cpp:180-214) run
// sequentially by one warp in the reference's order, only to learn which
// constraint's revision empties a domain first: the constraint whose weight
// the dom/wdeg order raises (src/AC3.cpp:122-128). Used for the nodes whose
// parallel fixpoint failed. Binary networks: variable x's incidences in the
// CSR are in increasing constraint order (the reference's subscription
// order, src/Network.cpp:402-403), arc_con[j] their constraint ids; a
// constraint's scope is (bx, by). D: the node's domains before its edit
// (overwritten); assigned: the level's flags. op / var / val: the node's
// edit (root: every variable is an event; assign: D(var) = {val}; refute:
// val removed, no AC when D(var) empties). out[0]: the constraint, or -1.
// ---------------------------------------------------------------------------
// Every lane runs the same control flow on warp-uniform values (queue
// positions, stamps, the counter t); lane 0 writes the queue, flags and
// stamps, __syncwarp orders those writes before the next reads; a revision
// tests 32 values of y per ballot.
template <int WT>
__global__ void k_ac3_replay(DevNet N, const int* arc_con, const int* bx, const int* by, u64* D,
                             const uint8_t* assigned, int op, int var, int val, ReplayScratch R, int* out) {
  const int lane = threadIdx.x & 31;
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  for (int i = lane; i < N.n; i += 32) {
    R.stamp_var[i] = 0;
    R.inq[i] = 0;
  }
  for (int i = lane; i < N.nb; i += 32) R.stamp_tab[i] = 0;
  // The node's edit.
  if (op != kOpRoot && lane < WT) {
    u64& w = D[static_cast<size_t>(var) * WT + lane];
    if (op == kOpRefute)
      w &= ~((lane == (val >> 6)) ? (1ull << (val & 63)) : 0ull);
    else
      w = (lane == (val >> 6)) ? (1ull << (val & 63)) : 0ull;
  }
  __syncwarp();
  if (lane == 0) *out = -1;
  if (op == kOpRefute) {
    u64 dv[WT];
    load_dom_uniform<WT>(D + static_cast<size_t>(var) * WT, dv);
    u64 any = 0;
#pragma unroll
    for (int w = 0; w < WT; ++w) any |= dv[w];
    if (!any) return;  // MAC::enforce does not call AC on an emptied domain (src/MAC.cpp:153-154)
  }
  const int qcap = N.n + 1;
  int qh = 0, qt = 0;
  unsigned long long t = 0;
  auto insert = [&](int v) {
    const bool fresh = !R.inq[v];  // uniform: read after the last __syncwarp
    __syncwarp();
    if (lane == 0) {
      if (fresh) {
        R.q[qt] = v;
        R.inq[v] = 1;
      }
      R.stamp_var[v] = t + 1;
    }
    if (fresh) qt = (qt + 1) % qcap;
    ++t;
    __syncwarp();
  };
  if (op == kOpRoot) {
    for (int v = 0; v < N.n; ++v) insert(v);
  } else {
    insert(var);
  }
  // Each pop follows an insert, and every insert after the events follows a
  // removal, so the loop ends; the cap only guards against a broken network.
  long long guard = N.total_values + N.n + 2;
  while (qh != qt && guard-- > 0) {
    const int x = R.q[qh];
    qh = (qh + 1) % qcap;
    __syncwarp();
    if (lane == 0) R.inq[x] = 0;
    __syncwarp();
    const int a0 = N.arc_start[x], a1 = N.arc_start[x + 1];
    for (int j = a0; j < a1; ++j) {
      const int c = arc_con[j];
      if (!(R.stamp_var[x] > R.stamp_tab[c])) continue;
      const Arc A = N.arcs[j];  // out of x: A.z the other variable
      const int sc[2] = {bx[c], by[c]};
      const int not_x = sc[0] == x ? sc[1] : sc[0];
      for (int k = 0; k < 2; ++k) {
        const int y = sc[k];
        if (assigned[y]) continue;
        const int other = sc[1 - k];
        // Read now: revising the first scope variable may have stamped it.
        const bool aa = R.stamp_var[not_x] > R.stamp_tab[c];
        if (y == x && !aa) continue;
        // revise(arc(c, y)): the values of y without a support in D(other).
        const u32 rows = (y == x) ? A.yz : A.zy;
        u64 dy[WT], dw[WT], rm[WT];
        load_dom_uniform<WT>(D + static_cast<size_t>(y) * WT, dy);
        load_dom_uniform<WT>(D + static_cast<size_t>(other) * WT, dw);
#pragma unroll
        for (int w = 0; w < WT; ++w) rm[w] = 0;
        valuewise_removals_seq<WT>(N, rows, dw, dy, rm);
        bool changed = false, empty = true;
#pragma unroll
        for (int w = 0; w < WT; ++w) {
          changed |= rm[w] != 0;
          empty &= (dy[w] & ~rm[w]) == 0;
        }
        if (!changed) continue;
        if (lane < WT) D[static_cast<size_t>(y) * WT + lane] = sel<WT>(dy, lane) & ~sel<WT>(rm, lane);
        __syncwarp();
        if (empty) {
          if (lane == 0) *out = c;
          return;
        }
        insert(y);
      }
      ++t;
      __syncwarp();
      if (lane == 0) R.stamp_tab[c] = t;
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------------------
// Small kernels.
// ---------------------------------------------------------------------------
// Live (x, a) pairs of a level, one warp per variable: ballot of the live
// flags, lane offsets by prefix popcount, one atomic per 32 values.
// The work list of a sweep (block vb of vg blocks of the body): one warp per
// variable appends its live values; with snap, the sweep-start domains are
// copied too.
template <int WT>
__device__ __forceinline__ void build_work_body(const DevNet& N, const u64* dom, int2* work, int* nwork, int4* tiles,
                                                int* ntiles, u64* snap, int vb, int vg) {
  const int lane = threadIdx.x & 31;
  const int gw = (vb * blockDim.x + threadIdx.x) >> 5;
  const int nw = (vg * blockDim.x) >> 5;
  if (snap)  // the sweep-start domains, for the tiled sweep
    for (size_t i = vb * static_cast<size_t>(blockDim.x) + threadIdx.x; i < static_cast<size_t>(N.n) * WT;
         i += static_cast<size_t>(vg) * blockDim.x)
      snap[i] = dom[i];
  for (int x = gw; x < N.n; x += nw) {
    const int ds = N.dsize[x];
    for (int base = 0; base < ds; base += 32) {
      const u64 word = dom[static_cast<size_t>(x) * WT + (base >> 6)];
      const u32 bits = static_cast<u32>(word >> (base & 32));
      if (bits == 0) continue;
      int b0 = 0;
      if (lane == 0) {
        b0 = atomicAdd(nwork, __popc(bits));
        if (tiles) tiles[atomicAdd(ntiles, 1)] = make_int4(x, base, b0, static_cast<int>(bits));
      }
      b0 = __shfl_sync(kFull, b0, 0);
      if ((bits >> lane) & 1u) work[b0 + __popc(bits & ((1u << lane) - 1u))] = make_int2(x, base + lane);
    }
  }
}

template <int WT>
__global__ void k_build_work(DevNet N, const u64* dom, int2* work, int* nwork, int4* tiles, int* ntiles, u64* snap) {
  build_work_body<WT>(N, dom, work, nwork, tiles, ntiles, snap, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------
// k_sac_tile: the singleton tests of 32 values of one variable x at once,
// lane l of every warp standing for branch (x, base + l).
//
// On an AC-closed level, the fixpoint of branch (x, a) is reached after two
// rounds unless round two removes something: round one only shrinks the
// neighbours y of x to D0(y) & R[x=a -> y]; round two revises every arc
// (z <- y) out of those neighbours. This kernel computes round one for all 32
// branches into shared memory, then only tests round two, one lane per arc:
// a value v of z can lose every support in branch b only if its support count
// in D0(y) is at most the number of values b's round one removed from D0(y),
// so the lane tests just those (branch, value) pairs, taking v from the arc's
// weak-support list; an arc whose list does not reach far enough for some
// branch is revised value-wise by the whole warp for those branches. A branch
// whose round two would remove nothing is consistent; one whose round two
// empties a domain is not; any other branch (round two removes values) is
// handed to the general kernel, which computes its fixpoint in full. Arcs
// back into x need no test: x's single value keeps a support in every
// non-empty D_a(y) by construction.
// ---------------------------------------------------------------------------
template <int WT>
__device__ __forceinline__ int pop_low(u64& m, int word) {
  if (!m) return -1;
  const int b = __ffsll(static_cast<long long>(m)) - 1;
  m &= m - 1;
  return word * 64 + b;
}

// One tile: branches (x, base + l) for the live lanes l of `live`; work index
// of the first live lane is b0. slot_of must be all -1 on entry and is left so;
// s_fail / s_deep must be zero and visible to the whole CTA on entry. Ends
// with the CTA synchronised.
template <int WT>
__device__ __forceinline__ void tile_one(const DevNet& N, u64* root, const u64* snap, const u32* weak, bool gs, int x,
                                         int base, int b0,
                                         u32 live, uint8_t* ok, int* deep, int* ndeep, int slot_cap, u64* T,
                                         int4* nbr, int* slot_of, u32& s_fail, u32& s_deep, int& s_next, int* s_rem, u32* s_msk, u64& c_rev,
                                         u64& c_rows, u64& c_done) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  {
    const int a0 = N.arc_start[x], deg = N.arc_start[x + 1] - a0;
    const bool fits = deg <= slot_cap;
    if (fits) {
      // Round one: slots for the distinct neighbours, D_a(y) = D0(y) & rows.
      for (int i = threadIdx.x; i < deg; i += blockDim.x) atomicCAS(&slot_of[N.arcs[a0 + i].z], -1, i);
      __syncthreads();
      // The first arc to each neighbour z writes D_a(z) = D0(z) & row(x = a)
      // (lanes without a branch keep D0(z)); further constraints on the same
      // pair, if any, AND their rows in afterwards.
      // Lane 0 also records the neighbour for round two: z, its arc range
      // and |D0(z)| in the sweep-start snapshot (-1: a repeated neighbour).
      bool dup = false;
      for (int i = warp; i < deg; i += nwarps) {
        const Arc A = N.arcs[a0 + i];
        if (slot_of[A.z] != i) {
          dup = true;
          if (lane == 0) nbr[i] = make_int4(-1, 0, 0, 0);
          continue;
        }
        if (lane == 0) {
          int c = 0;
#pragma unroll
          for (int w = 0; w < WT; ++w) c += __popcll(__ldg(snap + static_cast<size_t>(A.z) * WT + w));
          nbr[i] = make_int4(A.z, N.arc_start[A.z], N.arc_start[A.z + 1], c);
        }
        u64 d[WT], r[WT];
#pragma unroll
        for (int w = 0; w < WT; ++w) d[w] = root[static_cast<size_t>(A.z) * WT + w];
        if ((live >> lane) & 1u) {
          load_row<WT>(N.rel, A.yz + static_cast<size_t>(base + lane) * WT, r);
#pragma unroll
          for (int w = 0; w < WT; ++w) d[w] &= r[w];
        }
#pragma unroll
        for (int w = 0; w < WT; ++w) T[(static_cast<size_t>(i) * 32 + lane) * WT + w] = d[w];
      }
      if (__syncthreads_or(dup)) {
        for (int i = warp; i < deg; i += nwarps) {
          const Arc A = N.arcs[a0 + i];
          const int s = slot_of[A.z];
          if (s == i || !((live >> lane) & 1u)) continue;
          u64 r[WT];
          load_row<WT>(N.rel, A.yz + static_cast<size_t>(base + lane) * WT, r);
#pragma unroll
          for (int w = 0; w < WT; ++w) atomicAnd(&T[(static_cast<size_t>(s) * 32 + lane) * WT + w], r[w]);
        }
        __syncthreads();
      }
      for (int k = threadIdx.x; k < deg * 32; k += blockDim.x) {
        const int i = k >> 5, l = k & 31;
        if (slot_of[N.arcs[a0 + i].z] != i || !((live >> l) & 1u)) continue;
        u64 any = 0;
#pragma unroll
        for (int w = 0; w < WT; ++w) any |= T[(static_cast<size_t>(i) * 32 + l) * WT + w];
        if (!any) atomicOr(&s_fail, 1u << l);
      }
      if (threadIdx.x == 0) s_next = 0;
      __syncthreads();
      // Round two, tested only; warps take neighbours y dynamically (their
      // costs differ), so fewer wait at the barrier that ends the tile. Lane j
      // of a warp owns arc jb + j out of y. A value v of z can lose every
      // support in branch b only if its support count in D0(y) is at most the
      // number of values of D0(y) that b's round one removed (pigeonhole), so a
      // lane tests just those (branch, value) pairs, taking v from the arc's
      // weak list in increasing count order: one row load per value serves all
      // its branches. Branches that reach past the end of an arc's list need
      // the whole arc: the warp revises such arcs together, one lane per branch.
      int* rem = s_rem + warp * 32;  // removed count of each open branch, -1 if closed
      u32* msk = s_msk + warp * 32;  // threshold masks of the current chunk
      for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(&s_next, 1);
        item = __shfl_sync(kFull, item, 0);
        // Two items per neighbour, alternate 32-arc chunks: every first half,
        // then the (shorter) second halves, so a tile ends on small items.
        if (item >= 2 * deg) break;
        const int half = item >= deg ? 1 : 0;
        const int s = item - half * deg;
        const int4 ny = nbr[s];
        if (ny.x < 0) continue;
        const int y0 = ny.y, y1 = ny.z;
        const u64* Ty = T + static_cast<size_t>(s) * 32 * WT;  // D_b(y) at Ty + b * WT
        u64 dy[WT];
        int removed = ny.w;  // values of D0(y) this lane's round one removed
#pragma unroll
        for (int w = 0; w < WT; ++w) {
          dy[w] = Ty[lane * WT + w];
          removed -= __popcll(dy[w]);
        }
        for (int jb = y0 + 32 * half; jb < y1; jb += 64) {
          // Branches still open (live, not failed, not handed over), warp-uniform.
          const u32 done_m = __shfl_sync(kFull, *reinterpret_cast<volatile u32*>(&s_fail) |
                                                    *reinterpret_cast<volatile u32*>(&s_deep), 0);
          const u32 open = live & ~done_m;
          if (!open) break;
          const int r_own = ((open >> lane) & 1u) ? removed : -1;
          const int jl = jb + lane;
          const u32* wl = weak ? weak + static_cast<size_t>(jl) * kWeakStride : nullptr;
          Arc A{};
          bool arc_in = false;
          uint4 wv = make_uint4(0u, 0u, 0u, 0u);  // next count, entries 0..2 (zeros without lists)
          if (jl < y1) {
            A = N.arcs[jl];
            if (wl) wv = __ldg(reinterpret_cast<const uint4*>(wl));
            arc_in = A.z != x;
          }
          // Lowest support count among the arc's values (0 without lists:
          // every open branch then needs the whole arc).
          const int c0 = static_cast<int>(wv.y >> 16);
          const u32 arcs_m = __ballot_sync(kFull, arc_in);
          if (lane == 0) c_rev += __popc(arcs_m);
          const int cmin = __reduce_min_sync(kFull, arc_in ? c0 : 0x7fffffff);
          const int rtop = __reduce_max_sync(kFull, r_own);
          if (rtop < cmin) continue;  // no open branch reaches any arc of the chunk
          // ge(t): the open branches whose removed count is at least t, tabled
          // for t in [cmin, cmin + 31] (no count of the chunk is below cmin).
          __syncwarp();
          rem[lane] = r_own;
          const int thi = min(rtop, cmin + 31);
          for (int t = cmin; t <= thi; ++t) {
            const u32 mt = __ballot_sync(kFull, r_own >= t);
            if (lane == 0) msk[t - cmin] = mt;
          }
          __syncwarp();
          auto ge = [&](int t) -> u32 {
            if (t > rtop) return 0u;
            if (t - cmin < 32) return msk[t - cmin];
            u32 m = 0;
            for (int b = 0; b < 32; ++b)
              if (rem[b] >= t) m |= 1u << b;
            return m;
          };
          u32 fm = 0;  // branches that need this lane's arc in full
          const u32 bm = arc_in ? ge(c0) : 0u;
          if (bm) {
            const u32 fmask = ge(static_cast<int>(wv.x >> 16));  // past the list's end
            fm = bm & fmask;
            const u32 wm = bm & ~fmask;
            if (wm) {
              // Rows of the first kPre entries in one wave of loads, with D(z).
              constexpr int kPre = WT <= 2 ? 3 : 1;
              const u32 ent[3] = {wv.y, wv.z, wv.w};
              u32 pk[kPre];  // branches that test entry p
              u64 pre[kPre][WT];
#pragma unroll
              for (int p = 0; p < kPre; ++p) {
                pk[p] = wm & ge(static_cast<int>(ent[p] >> 16));
                if (pk[p]) {
                  load_row<WT>(N.rel, A.zy + static_cast<size_t>(ent[p] & 0xffffu) * WT, pre[p]);
                } else {
#pragma unroll
                  for (int w = 0; w < WT; ++w) pre[p][w] = 0;
                }
              }
              const int sz = slot_of[A.z];
              const u64* Tz = T + static_cast<size_t>(sz < 0 ? 0 : sz) * 32 * WT;  // D_b(z) if z neighbours x
              u64 cz[WT];  // D(z) otherwise, the same in every branch
#pragma unroll
              for (int w = 0; w < WT; ++w) cz[w] = sz < 0 ? root[static_cast<size_t>(A.z) * WT + w] : 0ull;
              u32 hitm = 0;  // branches in which some listed value of z loses every support
              u64 nrows = 0;
              // Entry e (row r) in the branches bk that reach its count.
              auto test = [&](u32 e, u32 bk, const u64 (&r)[WT]) {
                ++nrows;
                const int v = static_cast<int>(e & 0xffffu);
                const int vw = v >> 6;
                const u64 vbit = 1ull << (v & 63);
                const bool in_cz = (sel<WT>(cz, vw) & vbit) != 0;
                for (u32 m = bk; m; m &= m - 1) {
                  const int b = __ffs(m) - 1;
                  if (!(sz < 0 ? in_cz : (Tz[b * WT + vw] & vbit) != 0)) continue;
                  u64 t[WT];
                  load_sh<WT>(Ty + b * WT, t);
                  u64 hit = 0;
#pragma unroll
                  for (int w = 0; w < WT; ++w) hit |= r[w] & t[w];
                  if (!hit) hitm |= 1u << b;
                }
              };
#pragma unroll
              for (int p = 0; p < kPre; ++p)
                if (pk[p]) test(ent[p], pk[p], pre[p]);
              // Counts increase along the list: once an entry reaches no
              // branch, no later one does.
              if (pk[kPre - 1]) {
                for (int k = kPre; k < kWeakK; ++k) {
                  const u32 e = __ldg(wl + 1 + k);
                  const u32 bk = wm & ge(static_cast<int>(e >> 16));
                  if (!bk) break;
                  u64 r[WT];
                  load_row<WT>(N.rel, A.zy + static_cast<size_t>(e & 0xffffu) * WT, r);
                  test(e, bk, r);
                }
              }
              // Rare: round two removes values of z in branch b. A wipeout of
              // D_b(z) fails b, anything less hands it over.
              for (u32 m = hitm; m; m &= m - 1) {
                const int b = __ffs(m) - 1;
                const int rb = rem[b];
                int unsup = 0, size = 0;
#pragma unroll
                for (int w = 0; w < WT; ++w) size += __popcll(sz < 0 ? cz[w] : Tz[b * WT + w]);
                for (int k = 0; k < kWeakK; ++k) {
                  const u32 e = __ldg(wl + 1 + k);
                  if (static_cast<int>(e >> 16) > rb) break;
                  const int v = static_cast<int>(e & 0xffffu);
                  const u64 vbit = 1ull << (v & 63);
                  if (!((sz < 0 ? sel<WT>(cz, v >> 6) : Tz[b * WT + (v >> 6)]) & vbit)) continue;
                  u64 row[WT];
                  load_row<WT>(N.rel, A.zy + static_cast<size_t>(v) * WT, row);
                  ++nrows;
                  u64 hit = 0;
#pragma unroll
                  for (int w = 0; w < WT; ++w) hit |= row[w] & Ty[b * WT + w];
                  if (!hit) ++unsup;
                }
                atomicOr(unsup < size ? &s_deep : &s_fail, 1u << b);
              }
              c_rows += nrows;
            }
          }
          // Arcs whose list does not cover some branch: the warp revises each
          // value-wise, lane l holding the rows of the values l, l + 32, ...
          // of z (one wave of loads), and tests them against D_b(y) of every
          // such branch b: v in D_b(z) keeps a support iff its row meets D_b(y).
          for (u32 fullm = __ballot_sync(kFull, fm != 0); fullm; fullm &= fullm - 1) {
            const int k = __ffs(fullm) - 1;
            const u32 fmk = __shfl_sync(kFull, fm, k);
            const Arc Af = N.arcs[jb + k];
            const int sz = slot_of[Af.z];
            const u64* Tz = T + static_cast<size_t>(sz < 0 ? 0 : sz) * 32 * WT;
            u64 cz[WT], un[WT];  // D(z) if z is no neighbour of x; the values some such branch has
#pragma unroll
            for (int w = 0; w < WT; ++w) un[w] = cz[w] = sz < 0 ? root[static_cast<size_t>(Af.z) * WT + w] : 0ull;
            if (sz >= 0) {
              for (u32 m = fmk; m; m &= m - 1) {
                const int b = __ffs(m) - 1;
#pragma unroll
                for (int w = 0; w < WT; ++w) un[w] |= Tz[b * WT + w];
              }
            }
            u32 stillm = 0, leftm = 0;  // branches with an unsupported / a supported value of z
            int loaded = 0;
            constexpr int kG = WT <= 2 ? 2 * WT : 2;  // rows in flight per lane
#pragma unroll
            for (int h0 = 0; h0 < 2 * WT; h0 += kG) {
              u64 r[kG][WT];
              bool need[kG];
#pragma unroll
              for (int g = 0; g < kG; ++g) {
                const int h = h0 + g;
                need[g] = (sel<WT>(un, h >> 1) >> ((h & 1) * 32 + lane)) & 1ull;
                if (need[g]) {
                  load_row<WT>(N.rel, Af.zy + static_cast<size_t>(h * 32 + lane) * WT, r[g]);
                } else {
#pragma unroll
                  for (int w = 0; w < WT; ++w) r[g][w] = 0;
                }
                loaded += __popc(__ballot_sync(kFull, need[g]));
              }
              for (u32 m = fmk; m; m &= m - 1) {
                const int b = __ffs(m) - 1;
                u64 t[WT];
                load_sh<WT>(Ty + b * WT, t);
#pragma unroll
                for (int g = 0; g < kG; ++g) {
                  const int h = h0 + g;
                  const u64 curw = sz < 0 ? sel<WT>(cz, h >> 1) : Tz[b * WT + (h >> 1)];
                  const bool vin = (curw >> ((h & 1) * 32 + lane)) & 1ull;
                  u64 hit = 0;
#pragma unroll
                  for (int w = 0; w < WT; ++w) hit |= r[g][w] & t[w];
                  if (__ballot_sync(kFull, vin && hit == 0)) stillm |= 1u << b;
                  if (__ballot_sync(kFull, vin && hit != 0)) leftm |= 1u << b;
                }
              }
            }
            if (lane == 0) {
              c_rows += loaded;
              for (u32 m = stillm; m; m &= m - 1) {
                const int b = __ffs(m) - 1;
                atomicOr(((leftm >> b) & 1u) ? &s_deep : &s_fail, 1u << b);
              }
            }
          }
        }
      }
      __syncthreads();
      for (int i = threadIdx.x; i < deg; i += blockDim.x) slot_of[N.arcs[a0 + i].z] = -1;
    }
    // Verdicts: warp 0 writes them; handed-over branches go to the deep list.
    if (warp == 0) {
      const bool is_live = (live >> lane) & 1u;
      const u32 failm = *reinterpret_cast<volatile u32*>(&s_fail);
      const u32 deepm = fits ? *reinterpret_cast<volatile u32*>(&s_deep) : live;
      const bool f = is_live && ((failm >> lane) & 1u);
      if (gs && f)  // early removal at the level: later branches of the sweep start without it
        atomicAnd(root + static_cast<size_t>(x) * WT + ((base + lane) >> 6), ~(1ull << ((base + lane) & 63)));
      const bool d = is_live && !f && ((deepm >> lane) & 1u);
      const int b = b0 + __popc(live & ((1u << lane) - 1u));
      const u32 dm = __ballot_sync(kFull, d);
      int db = 0;
      if (lane == 0 && dm) db = atomicAdd(ndeep, __popc(dm));
      db = __shfl_sync(kFull, db, 0);
      if (d) deep[db + __popc(dm & ((1u << lane) - 1u))] = b;
      if (is_live && !d) ok[b] = f ? 0 : 1;
      if (lane == 0) c_done += __popc(live & ~dm);
    }
    __syncthreads();
  }
}

// Weak-support lists for the root domains: per directional arc j (revise z
// against y), at word 0 the count of the (kWeakK+1)-th weakest value as
// count << 16 | 0xffff (0xffffffff: none), then the kWeakK values v of D(z)
// with the fewest supports |row_zy(v) & D(y)| in increasing (count, v) order
// as count << 16 | v (0xffffffff past the end), then padding. One warp per
// arc; the smallest keys are taken by repeated warp minima.
template <int WT>
__device__ void weak_list_arc(const DevNet& N, const u64* root, const Arc A, int j, u32* weak) {
  const int lane = threadIdx.x & 31;
  const int z = A.z, dz = N.dsize[z];
  // D(y) (y = the arc's source) and D(z), both loaded before either is
  // broadcast (one word per lane), so the two loads overlap.
  const u64 wy = lane < WT ? vload(root + static_cast<size_t>(A.src) * WT + lane) : 0ull;
  const u64 wz = lane < WT ? vload(root + static_cast<size_t>(z) * WT + lane) : 0ull;
  u64 dy[WT], d0z[WT];
#pragma unroll
  for (int w = 0; w < WT; ++w) {
    dy[w] = __shfl_sync(kFull, wy, w);
    d0z[w] = __shfl_sync(kFull, wz, w);
  }
  u32 key[2 * WT];
#pragma unroll
  for (int t = 0; t < 2 * WT; ++t) {
    const int v = t * 32 + lane;
    key[t] = 0xffffffffu;
    if (v < dz && ((sel<WT>(d0z, v >> 6) >> (v & 63)) & 1ull)) {
      u64 r[WT];
      load_row<WT>(N.rel, A.zy + static_cast<size_t>(v) * WT, r);
      int c = 0;
#pragma unroll
      for (int w = 0; w < WT; ++w) c += __popcll(r[w] & dy[w]);
      key[t] = (static_cast<u32>(c) << 16) | static_cast<u32>(v);
    }
  }
  u32* out = weak + static_cast<size_t>(j) * kWeakStride;
  if (lane > kWeakK && lane < kWeakStride) out[lane] = 0xffffffffu;  // padding
  // Writes the k-th smallest key m; true once the keys are exhausted.
  auto emit = [&](int k, u32 m) -> bool {
    if (lane == 0) {
      if (k < kWeakK)
        out[1 + k] = m;
      else
        out[0] = m | 0xffffu;
    }
    if (m != 0xffffffffu) return false;
    if (lane == 0) {
      for (int r = k + 1; r < kWeakK; ++r) out[1 + r] = 0xffffffffu;
      out[0] = 0xffffffffu;
    }
    return true;
  };
  if constexpr (WT <= 4) {
    // Each lane's keys in increasing order (odd-even transposition); a step
    // then takes the warp minimum of the lanes' first keys, and the lane that
    // owns it (keys are distinct) moves on to its next key.
#pragma unroll
    for (int i = 0; i < 2 * WT; ++i) {
#pragma unroll
      for (int t = i & 1; t + 1 < 2 * WT; t += 2) {
        const u32 a = key[t], b = key[t + 1];
        key[t] = min(a, b);
        key[t + 1] = max(a, b);
      }
    }
    for (int k = 0; k <= kWeakK; ++k) {
      const u32 m = __reduce_min_sync(kFull, key[0]);
      if (emit(k, m)) break;
      if (key[0] == m) {
#pragma unroll
        for (int t = 0; t + 1 < 2 * WT; ++t) key[t] = key[t + 1];
        key[2 * WT - 1] = 0xffffffffu;
      }
    }
  } else {
    for (int k = 0; k <= kWeakK; ++k) {
      u32 m = key[0];
#pragma unroll
      for (int t = 1; t < 2 * WT; ++t) m = min(m, key[t]);
      m = __reduce_min_sync(kFull, m);
      if (emit(k, m)) break;
#pragma unroll
      for (int t = 0; t < 2 * WT; ++t)
        if (key[t] == m) key[t] = 0xffffffffu;
    }
  }
}

// Lists of all arcs of source variable y (one warp).
template <int WT>
__device__ void weak_lists_of(const DevNet& N, const u64* root, int y, u32* weak) {
  for (int j = N.arc_start[y]; j < N.arc_start[y + 1]; ++j) weak_list_arc<WT>(N, root, N.arcs[j], j, weak);
}

// Weak-support lists of every arc, one warp per arc (block vb of vg blocks of
// the body).
template <int WT>
__device__ __forceinline__ void weak_body(const DevNet& N, const u64* root, u32* weak, int vb, int vg) {
  const int gw = (vb * blockDim.x + threadIdx.x) >> 5;
  const int nw = (vg * blockDim.x) >> 5;
  const int narcs = N.arc_start[N.n];
  for (int j = gw; j < narcs; j += nw) weak_list_arc<WT>(N, root, N.arcs[j], j, weak);
}

// The sweep's work list and its weak-support lists in one launch: the first
// work_blocks blocks build the list (and the snapshot), the others the lists.
// Both read the level's domains, which nothing changes before the sweep.
template <int WT>
__global__ void k_work_and_weak(DevNet N, const u64* dom, int2* work, int* nwork, int4* tiles, int* ntiles, u64* snap,
                                u32* weak, int work_blocks) {
  pdl_wait();
  if (static_cast<int>(blockIdx.x) < work_blocks)
    build_work_body<WT>(N, dom, work, nwork, tiles, ntiles, snap, blockIdx.x, work_blocks);
  else
    weak_body<WT>(N, dom, weak, blockIdx.x - work_blocks, gridDim.x - work_blocks);
}

__device__ __forceinline__ void flush_tile_counts(KStats* st, u64 c_rev, u64 c_rows, u64 c_done) {
  Cnt cn;
  cn.rev = c_rev;
  cn.rows = c_rows;
  flush_counts(st, cn);
  if (threadIdx.x == 0 && c_done) {
    atomicAdd(&st->fixpoints, c_done);
    atomicAdd(&st->branches, c_done);
    atomicMax(&st->rounds_max, 2);
  }
}

template <int WT>
__global__ void __launch_bounds__(256, WT <= 2 ? 5 : 1) k_sac_tile(DevNet N, u64* root, const u64* snap,
                                                                   const int4* tiles, const int* ntiles, int* tcursor,
                                                                   uint8_t* ok, int* deep, int* ndeep, int slot_cap,
                                                                   KStats* st, const u32* weak) {
  pdl_wait();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  u64* T = reinterpret_cast<u64*>(smem_raw);  // [slot_cap][32][WT]
  int4* nbr = reinterpret_cast<int4*>(smem_raw + static_cast<size_t>(slot_cap) * 32 * WT * 8);  // [slot_cap]
  int* slot_of = reinterpret_cast<int*>(nbr + slot_cap);  // [n]
  __shared__ int s_t;
  __shared__ u32 s_fail, s_deep;
  __shared__ int s_next;
  __shared__ int s_rem[256];  // 256-thread CTAs: 32 per warp
  __shared__ u32 s_msk[256];
  const int total = *ntiles;
  for (int i = threadIdx.x; i < N.n; i += blockDim.x) slot_of[i] = -1;
  u64 c_rev = 0, c_rows = 0, c_done = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      s_t = atomicAdd(tcursor, 1);
      s_fail = 0;
      s_deep = 0;
    }
    __syncthreads();
    const int t = s_t;
    if (t >= total) break;
    const int4 tl = tiles[t];
    tile_one<WT>(N, root, snap ? snap : root, weak, snap != nullptr, tl.x, tl.y, tl.z, static_cast<u32>(tl.w), ok,
                 deep, ndeep, slot_cap, T, nbr, slot_of, s_fail, s_deep, s_next, s_rem, s_msk, c_rev, c_rows, c_done);
  }
  flush_tile_counts(st, c_rev, c_rows, c_done);
}

// With out: the last block to finish (counted on done, which it resets)
// copies the round's nst stats slots into host-mapped memory and, with
// dom_out, when the sweep removed nothing (the level is the closure), the
// level's dom_words words too.
__global__ void k_commit(int W, const int2* work, const int* nwork, const uint8_t* ok, u64* dom, int* evt, int* nevt,
                         u32* evt_fb, KStats* st, unsigned* done, KStats* out, int nst, u64* dom_out,
                         size_t dom_words) {
  pdl_wait();
  const int total = *nwork;
  u64 removed = 0;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < total; b += gridDim.x * blockDim.x) {
    if (ok[b]) continue;
    const int2 xa = work[b];
    atomicAnd(dom + static_cast<size_t>(xa.x) * W + (xa.y >> 6), ~(1ull << (xa.y & 63)));
    ++removed;
    const u32 bit = 1u << (xa.x & 31);
    if (!(atomicOr(evt_fb + (xa.x >> 5), bit) & bit)) evt[atomicAdd(nevt, 1)] = xa.x;
  }
  if (removed) {
    atomicAdd(&st->removed, removed);
    atomicAdd(&st->deletions, removed);
  }
  if (!out) return;
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  constexpr int kw = static_cast<int>(sizeof(KStats) / sizeof(int));
  const int* a = reinterpret_cast<const int*>(st);
  int* b = reinterpret_cast<int*>(out);
  for (int i = threadIdx.x; i < nst * kw; i += blockDim.x) b[i] = __ldcg(a + i);
  if (dom_out && __ldcg(&st->removed) == 0)
    for (size_t i = threadIdx.x; i < dom_words; i += blockDim.x) dom_out[i] = __ldcg(dom + i);
  __threadfence_system();
  if (threadIdx.x == 0) *done = 0u;
}

// 32x32 bit-matrix transpose across a warp: lane r holds row r (bit c =
// element (r, c)); afterwards lane r holds column r. Five butterfly steps
// swap the off-diagonal k x k blocks between lanes r and r ^ k.
__device__ __forceinline__ u32 warp_transpose32(u32 x) {
  const int lane = threadIdx.x & 31;
  const u32 masks[5] = {0x0000ffffu, 0x00ff00ffu, 0x0f0f0f0fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    const int k = 16 >> i;
    const u32 m = masks[i];
    const u32 y = __shfl_xor_sync(kFull, x, k);
    x = (lane & k) ? ((x & ~m) | ((y >> k) & m)) : ((x & m) | ((y << k) & ~m));
  }
  return x;
}

// B block of constraint c (rows of y values over x values) from its A block,
// one warp per (c, 32 y values b): for each 32-value group g of x, the lanes
// load the 32-bit slices [bb, bb + 32) of x rows g*32 + lane, transpose them
// in registers, and lane j keeps the slice g of y row bb + j; each y row is
// then written whole (2W u32 words) by its lane.
template <int WT>
__global__ void k_transpose(DevNet N, u64* rel, const int* bx, const int* by, const int64_t* offA,
                            const int64_t* offB, int chunks) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int item = gw; item < N.nb * chunks; item += nw) {
    const int c = item / chunks, bb = (item % chunks) * 32;
    const int dx = N.dsize[bx[c]], dy = N.dsize[by[c]];
    if (bb >= dy) continue;
    const u64* A = rel + offA[c];
    u32 out[2 * WT];
#pragma unroll
    for (int g = 0; g < 2 * WT; ++g) {
      const int a = g * 32 + lane;
      u32 slice = 0;
      if (a < dx) slice = static_cast<u32>(A[static_cast<int64_t>(a) * WT + (bb >> 6)] >> (bb & 32));
      out[g] = (g * 32 < dx) ? warp_transpose32(slice) : 0u;
    }
    const int b = bb + lane;
    if (b < dy) {
      u32* row = reinterpret_cast<u32*>(rel + offB[c] + static_cast<int64_t>(b) * WT);
#pragma unroll
      for (int g = 0; g < 2 * WT; ++g) row[g] = out[g];
    }
  }
}

// A blocks of seeded random relations generated on the device with the same
// counter-based relation_word as the host generator (cp_gen.h): one warp per
// constraint, lanes over its words.
__global__ void k_gen_rows(int nb, int W, const int* dsize, u64* rel, const int* bx, const int* by,
                           const int64_t* offA, const u64* cseed, const u32* thr) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int c = gw; c < nb; c += nw) {
    const int dx = dsize[bx[c]], dy = dsize[by[c]];
    const int wy = (dy + 63) / 64;
    const int total = dx * W;
    for (int i = lane; i < total; i += 32) {
      const int a = i / W, w = i % W;
      rel[offA[c] + i] = w < wy ? cpgen::relation_word(cseed[c], a, w, thr[c], dy) : 0ull;
    }
  }
}

template <int WT>
__global__ void k_popcount(int n, const u64* dom, int* sizes) {
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
    int s = 0;
#pragma unroll
    for (int w = 0; w < WT; ++w) s += __popcll(dom[static_cast<size_t>(x) * WT + w]);
    sizes[x] = s;
  }
}

__global__ void k_level_edit(int W, u64* dom, int var, int val, int op) {
  u64* dv = dom + static_cast<size_t>(var) * W;
  if (op == kOpAssign) {
    for (int w = 0; w < W; ++w) dv[w] = (w == (val >> 6)) ? (1ull << (val & 63)) : 0ull;
  } else {
    dv[val >> 6] &= ~(1ull << (val & 63));
  }
}

// ---------------------------------------------------------------------------
// Multi-instance batches: the same bodies, with the instance's DevNet copied
// into shared memory by the CTA that takes a work item of that instance.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void load_net(DevNet* dst, const DevNet* src) {
  if (threadIdx.x == 0) *dst = *src;
}

// Root or event AC of every listed instance; CTAs take instances in turn.
template <int WT, bool kTab>
__global__ void __launch_bounds__(512) k_batch_node(BatchDev B, int op, KStats* st, char* gscratch, size_t gstride) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_qlen[3], s_failed[2], s_failvar, s_err;
  __shared__ DevNet sN;
  char* base = gscratch ? gscratch + blockIdx.x * gstride : reinterpret_cast<char*>(smem_raw);
  const int count = *B.nact;
  if (threadIdx.x == 0) s_err = 0;
  Cnt cn;
  int rounds_max = 0;
  u64 done = 0;
  for (int i = blockIdx.x; i < count; i += gridDim.x) {
    const int inst = B.act_list[i];
    load_net(&sN, B.nets + inst);
    __syncthreads();
    const DevNet& N = sN;
    Fix F = make_cta_fix(N, base, s_qlen, s_failed, &s_failvar);
    const CtaLayout L = cta_layout(N);
    const size_t words = static_cast<size_t>(N.n) * WT;
    u64* dom = B.roots[inst];
    block_copy(F.D, dom, words);
    block_zero(reinterpret_cast<u32*>(base + L.fb0), (L.ts - L.fb0) / 4);
    if (N.nt) block_zero(reinterpret_cast<u32*>(F.tstamp), N.nt);
    if (threadIdx.x == 0) {
      s_qlen[0] = s_qlen[1] = s_qlen[2] = 0;
      s_failed[0] = s_failed[1] = 0;
    }
    __syncthreads();
    if (op == kOpRoot) {
      for (int z = threadIdx.x; z < N.n; z += blockDim.x) seed_var<WT>(N, F, z);
    } else {
      const int ne = B.nevt[inst];
      const int* ev = B.evt + B.var_base[inst];
      for (int j = threadIdx.x; j < ne; j += blockDim.x) seed_var<WT>(N, F, ev[j]);
    }
    __syncthreads();
    const int rounds = cta_fixpoint<WT, kTab, false>(N, F, cn, &s_err);
    rounds_max = max(rounds_max, rounds);
    block_copy(dom, F.D, words);
    if (threadIdx.x == 0 && (s_failed[0] | s_failed[1])) B.inc[inst] = 1;
    ++done;
    __syncthreads();
  }
  flush_counts(st, cn);
  if (threadIdx.x == 0) {
    atomicMax(&st->rounds_max, rounds_max);
    if (done) atomicAdd(&st->fixpoints, done);
    if (s_err) st->error = s_err;
  }
}

// Live pairs (and tiles) of every active instance; one warp per variable.
template <int WT>
__global__ void k_batch_build(BatchDev B, int with_tiles) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int g = gw; g < B.total_vars; g += nw) {
    const int inst = B.var_inst[g];
    if (!B.act[inst] || B.inc[inst]) continue;
    const int x = g - B.var_base[inst];
    const int ds = B.nets[inst].dsize[x];
    const u64* dom = B.roots[inst];
    const int tag = (inst << 16) | x;
    for (int base = 0; base < ds; base += 32) {
      const u64 word = dom[static_cast<size_t>(x) * WT + (base >> 6)];
      const u32 bits = static_cast<u32>(word >> (base & 32));
      if (bits == 0) continue;
      int b0 = 0;
      if (lane == 0) {
        b0 = atomicAdd(B.nwork, __popc(bits));
        if (with_tiles) B.tiles[atomicAdd(B.ntiles, 1)] = make_int4(tag, base, b0, static_cast<int>(bits));
      }
      b0 = __shfl_sync(kFull, b0, 0);
      if ((bits >> lane) & 1u) B.work[b0 + __popc(bits & ((1u << lane) - 1u))] = make_int2(tag, base + lane);
    }
  }
}

// The same lists for every active instance of a batch (instance i's lists at
// weak + weak_off[i]), one warp per variable.
template <int WT>
__global__ void k_batch_weak(BatchDev B) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int g = gw; g < B.total_vars; g += nw) {
    const int inst = B.var_inst[g];
    if (!B.act[inst] || B.inc[inst]) continue;
    weak_lists_of<WT>(B.nets[inst], B.roots[inst], g - B.var_base[inst], B.weak + B.weak_off[inst]);
  }
}

template <int WT>
// quota > 0: a CTA takes at most quota tiles and retires (the grid then
// covers every tile), so that CTAs of other streams get SMs between tiles.
__global__ void __launch_bounds__(256, WT <= 2 ? 4 : 1) k_batch_tile(BatchDev B, int slot_cap, int max_n, KStats* st, int quota) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  u64* T = reinterpret_cast<u64*>(smem_raw);
  int4* nbr = reinterpret_cast<int4*>(smem_raw + static_cast<size_t>(slot_cap) * 32 * WT * 8);
  int* slot_of = reinterpret_cast<int*>(nbr + slot_cap);
  __shared__ int s_t;
  __shared__ u32 s_fail, s_deep;
  __shared__ int s_next;
  __shared__ int s_rem[256];  // 256-thread CTAs: 32 per warp
  __shared__ u32 s_msk[256];
  __shared__ DevNet sN;
  const int total = *B.ntiles;
  for (int i = threadIdx.x; i < max_n; i += blockDim.x) slot_of[i] = -1;
  u64 c_rev = 0, c_rows = 0, c_done = 0;
  for (int taken = 0; quota == 0 || taken < quota; ++taken) {
    if (threadIdx.x == 0) {
      s_t = atomicAdd(B.tcursor, 1);
      s_fail = 0;
      s_deep = 0;
      if (s_t < total) sN = B.nets[B.tiles[s_t].x >> 16];
    }
    __syncthreads();
    const int t = s_t;
    if (t >= total) break;
    const int4 tl = B.tiles[t];
    const int inst = tl.x >> 16;
    tile_one<WT>(sN, B.roots[inst], B.snap ? B.snap + static_cast<size_t>(B.var_base[inst]) * WT : B.roots[inst],
                 B.weak ? B.weak + B.weak_off[inst] : nullptr, B.snap != nullptr, tl.x & 0xffff, tl.y, tl.z, static_cast<u32>(tl.w), B.ok, B.deep, B.ndeep,
                 slot_cap, T, nbr, slot_of, s_fail, s_deep, s_next, s_rem, s_msk, c_rev, c_rows, c_done);
  }
  flush_tile_counts(st, c_rev, c_rows, c_done);
}

// General singleton tests over the batch: all pairs, or the deep list.
template <int WT, bool kTab>
__global__ void __launch_bounds__(256) k_batch_sac(BatchDev B, int deep_only, KStats* st, char* gscratch,
                                                   size_t gstride, int quota) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_qlen[3], s_failed[2], s_failvar, s_err, s_b;
  __shared__ DevNet sN;
  char* base = gscratch ? gscratch + blockIdx.x * gstride : reinterpret_cast<char*>(smem_raw);
  const int total = deep_only ? *B.ndeep : *B.nwork;
  if (total == 0) return;  // an empty list: nothing to count either
  if (threadIdx.x == 0) s_err = 0;
  Cnt cn;
  int rounds_max = 0;
  u64 done = 0;
  for (int taken = 0; quota == 0 || taken < quota; ++taken) {
    if (threadIdx.x == 0) {
      s_b = atomicAdd(B.cursor, 1);
      if (s_b < total) {
        const int b = deep_only ? B.deep[s_b] : s_b;
        sN = B.nets[B.work[b].x >> 16];
      }
    }
    __syncthreads();
    const int i = s_b;
    if (i >= total) break;
    const int b = deep_only ? B.deep[i] : i;
    const int2 pr = B.work[b];
    const int inst = pr.x >> 16, x = pr.x & 0xffff, a = pr.y;
    const DevNet& N = sN;
    Fix F = make_cta_fix(N, base, s_qlen, s_failed, &s_failvar);
    const CtaLayout L = cta_layout(N);
    const size_t words = static_cast<size_t>(N.n) * WT;
    block_copy(F.D, B.roots[inst], words);
    block_zero(reinterpret_cast<u32*>(base + L.fb0), (L.ts - L.fb0) / 4);
    if (N.nt) block_zero(reinterpret_cast<u32*>(F.tstamp), N.nt);
    if (threadIdx.x == 0) {
      s_qlen[0] = s_qlen[1] = s_qlen[2] = 0;
      s_failed[0] = s_failed[1] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      u64* dv = F.D + static_cast<size_t>(x) * WT;
      for (int w = 0; w < WT; ++w) dv[w] = (w == (a >> 6)) ? (1ull << (a & 63)) : 0ull;
      append_var(F.q0, F.fb0, F.qlen, x);
    }
    __syncthreads();
    const int rounds = cta_fixpoint<WT, kTab, false>(N, F, cn, &s_err);
    rounds_max = max(rounds_max, rounds);
    if (threadIdx.x == 0) {
      const bool failed = (s_failed[0] | s_failed[1]) != 0;
      B.ok[b] = failed ? 0 : 1;
      if (failed && B.snap)  // early removal, as in k_sac
        atomicAnd(B.roots[inst] + static_cast<size_t>(x) * WT + (a >> 6), ~(1ull << (a & 63)));
    }
    ++done;
    __syncthreads();
  }
  flush_counts(st, cn);
  if (threadIdx.x == 0) {
    atomicMax(&st->rounds_max, rounds_max);
    if (done) {
      atomicAdd(&st->fixpoints, done);
      atomicAdd(&st->branches, done);
    }
    if (s_err) st->error = s_err;
  }
}

// Removes failed pairs from their instance's level; collects changed
// variables per instance.
__global__ void k_batch_commit(BatchDev B, int W, KStats* st) {
  const int total = *B.nwork;
  u64 removed = 0;
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < total; b += gridDim.x * blockDim.x) {
    if (B.ok[b]) continue;
    const int2 pr = B.work[b];
    const int inst = pr.x >> 16, x = pr.x & 0xffff, a = pr.y;
    atomicAnd(B.roots[inst] + static_cast<size_t>(x) * W + (a >> 6), ~(1ull << (a & 63)));
    atomicAdd(&B.removed[inst], 1);
    ++removed;
    const int g = B.var_base[inst] + x;
    const u32 bit = 1u << (g & 31);
    if (!(atomicOr(B.evt_fb + (g >> 5), bit) & bit)) B.evt[B.var_base[inst] + atomicAdd(&B.nevt[inst], 1)] = x;
  }
  if (removed) {
    atomicAdd(&st->removed, removed);
    atomicAdd(&st->deletions, removed);
  }
}

// Sweep-start copy of every active member's working domains into B.snap.
__global__ void k_batch_snap(BatchDev B, int W) {
  for (int i = blockIdx.x; i < B.k; i += gridDim.x) {
    if (!B.act[i] || B.inc[i]) continue;
    const size_t words = static_cast<size_t>(B.nets[i].n) * W;
    const u64* src = B.roots[i];
    u64* dst = B.snap + static_cast<size_t>(B.var_base[i]) * W;
    for (size_t j = threadIdx.x; j < words; j += blockDim.x) dst[j] = src[j];
  }
}

// Copies level (batch level + delta) of every member onto the batch level,
// one CTA per member in turn.
// Each instance's working level := level src_level of its own stack (a
// no-op where they coincide).
__global__ void k_batch_copy(BatchDev B, int W, int src_level) {
  for (int i = blockIdx.x; i < B.k; i += gridDim.x) {
    const size_t words = static_cast<size_t>(B.nets[i].n) * W;
    u64* dst = B.roots[i];
    const u64* src = B.bases[i] + static_cast<size_t>(src_level) * words;
    if (src == dst) continue;
    for (size_t j = threadIdx.x; j < words; j += blockDim.x) dst[j] = src[j];
  }
}

// Edit e reduces variable var[e] of instance member[e] (group-local index) to
// the single value val[e] (the empty set if val[e] is not in the domain).
// Several edits may hit one variable: the words are ANDed atomically.
__global__ void k_batch_edit(BatchDev B, int W, int n_edit, const int* member, const int* var, const int* val) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_edit) return;
  u64* dom = B.roots[member[e]] + static_cast<size_t>(var[e]) * W;
  const int a = val[e];
  for (int w = 0; w < W; ++w) {
    const u64 keep = (w == (a >> 6)) ? (1ull << (a & 63)) : 0ull;
    atomicAnd(reinterpret_cast<unsigned long long*>(dom + w), static_cast<unsigned long long>(keep));
  }
}

// Working domains of every instance into one buffer at the caller's width:
// instance i's variable x, word w at out[out_off[i] + x * wuser[i] + w].
__global__ void k_batch_gather(BatchDev B, int W, u64* out) {
  for (int i = blockIdx.x; i < B.k; i += gridDim.x) {
    const int n = B.nets[i].n, wu = B.wuser[i];
    const u64* src = B.roots[i];
    u64* dst = out + B.out_off[i];
    const int words = n * wu;
    for (int j = threadIdx.x; j < words; j += blockDim.x) {
      const int x = j / wu, w = j - x * wu;
      dst[j] = src[static_cast<size_t>(x) * W + w];
    }
  }
}

// Next sweep's instances: initial = every consistent instance; otherwise the
// consistent instances whose last commit removed values. Warp-ballot
// compaction into act_list.
__global__ void k_batch_select(BatchDev B, int initial) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int base = gw * 32; base < B.k; base += nw * 32) {
    const int i = base + lane;
    bool on = false;
    if (i < B.k) {
      on = !B.inc[i] && (initial || B.removed[i] > 0);
      B.act[i] = on ? 1 : 0;
    }
    const u32 m = __ballot_sync(kFull, on);
    int b0 = 0;
    if (lane == 0 && m) b0 = atomicAdd(B.nact, __popc(m));
    b0 = __shfl_sync(kFull, b0, 0);
    if (on) B.act_list[b0 + __popc(m & ((1u << lane) - 1u))] = i;
  }
}

template <typename F>
cudaError_t dispatch_w(int W, F&& f) {
  switch (W) {
    case 1: return f(std::integral_constant<int, 1>{});
    case 2: return f(std::integral_constant<int, 2>{});
    case 4: return f(std::integral_constant<int, 4>{});
    case 8: return f(std::integral_constant<int, 8>{});
    default: return cudaErrorInvalidValue;
  }
}

// Dispatch on the domain width and on whether the network has tables
// (binary-only networks use kernels without the table path, which keeps
// their register count low).
template <typename F>
cudaError_t dispatch_wt(const DevNet& N, F&& f) {
  if (N.nt > 0) {
    switch (N.W) {
      case 1: return f(std::integral_constant<int, 1>{}, std::true_type{});
      case 2: return f(std::integral_constant<int, 2>{}, std::true_type{});
      case 4: return f(std::integral_constant<int, 4>{}, std::true_type{});
      case 8: return f(std::integral_constant<int, 8>{}, std::true_type{});
      default: return cudaErrorInvalidValue;
    }
  }
  return dispatch_w(N.W, [&](auto wt) { return f(wt, std::false_type{}); });
}

// Launches a kernel with programmatic stream serialisation (the kernel starts
// with pdl_wait()), so that its launch overlaps the end of the previous
// kernel on the stream, in direct launches and in captured graphs alike.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

template <typename K>
cudaError_t allow_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
}

}  // namespace

size_t cta_state_bytes(const DevNet& N) { return cta_layout(N).total; }

cudaError_t launch_node(const DevNet& N, u64* levels, int src, int dst, int op, int var, int val, const int* evt,
                        int nevt, KStats* st, uint8_t* ok_out, int block, void* gscratch, cudaStream_t s) {
  const size_t smem = gscratch ? 0 : cta_state_bytes(N);
  return dispatch_wt(N, [&](auto wt, auto tab) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    constexpr bool TB = decltype(tab)::value;
    cudaError_t e = allow_smem(k_node<WT, TB>, smem);
    if (e != cudaSuccess) return e;
    k_node<WT, TB><<<1, block, smem, s>>>(N, levels, src, dst, op, var, val, evt, nevt, st, ok_out,
                                      static_cast<char*>(gscratch));
    return cudaGetLastError();
  });
}

template <typename F>
cudaError_t dispatch_wtab(int W, bool tables, F&& f) {
  DevNet probe;
  probe.W = W;
  probe.nt = tables ? 1 : 0;
  return dispatch_wt(probe, f);
}

int mac_blocks_per_sm(int block, size_t smem) {
  int per_sm = 0;
  if (allow_smem(k_mac, smem) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mac, block, smem) != cudaSuccess) return 0;
  return per_sm;
}

cudaError_t launch_mac(const DevNet* nets, const MacJob* jobs, int njobs, int* cursor, MacOut* outs, int block,
                       int grid, size_t smem, void* gscratch, size_t gstride, long long slice_ns, cudaStream_t s) {
  const size_t dyn = gscratch ? 0 : smem;
  cudaError_t e = allow_smem(k_mac, dyn);
  if (e != cudaSuccess) return e;
  k_mac<<<grid, block, dyn, s>>>(nets, jobs, njobs, cursor, outs, static_cast<char*>(gscratch), gstride, slice_ns);
  return cudaGetLastError();
}

cudaError_t launch_ac3_replay(const DevNet& N, const int* arc_con, const int* bx, const int* by, u64* D,
                              const uint8_t* assigned, int op, int var, int val, ReplayScratch R, int* out,
                              cudaStream_t s) {
  return dispatch_w(N.W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    k_ac3_replay<WT><<<1, 32, 0, s>>>(N, arc_con, bx, by, D, assigned, op, var, val, R, out);
    return cudaGetLastError();
  });
}

int ac_front_max_blocks(const DevNet& N, int sm_count) {
  int per_sm = 0;
  cudaError_t e = dispatch_wt(N, [&](auto wt, auto tab) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    constexpr bool TB = decltype(tab)::value;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_ac_front<WT, TB>, kFrontBlock, 0);
  });
  if (e != cudaSuccess || per_sm < 1) return 0;
  return per_sm * sm_count;
}

static int front_tasks(const DevNet& N, int narcs) {
  int K = 1;
  dispatch_wt(N, [&](auto wt, auto) -> cudaError_t {
    K = FrontGroup<decltype(wt)::value>::K;
    return cudaSuccess;
  });
  return (narcs + K - 1) / K + N.nt;
}

int ac_front_blocks(const DevNet& N, int narcs, int sm_count) {
  const int most = ac_front_max_blocks(N, sm_count);
  if (most < 1) return 0;
  // One warp per task of a full round, at most every co-resident CTA.
  const int warps = kFrontBlock / 32;
  return std::max(1, std::min(most, (front_tasks(N, narcs) + warps - 1) / warps));
}

cudaError_t launch_ac_front(const DevNet& N, u64* level_dom, const int* evt, const int* nevt_dev, int nevt,
                            GridScratch G, KStats* st, int grid, cudaStream_t s) {
  return dispatch_wt(N, [&](auto wt, auto tab) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    constexpr bool TB = decltype(tab)::value;
    int first = 0;
    if (!evt) {
      // Round 0 as a plain launch, one warp per task.
      const int warps = kFrontBlock / 32;
      const int blocks = std::max(1, (front_tasks(N, 2 * N.nb) + warps - 1) / warps);
      cudaError_t e = launch_pdl(k_front_first<WT, TB>, dim3(blocks), dim3(kFrontBlock), 0, s, N, level_dom, G, st);
      if (e != cudaSuccess) return e;
      first = 1;
    }
    DevNet n2 = N;
    void* args[] = {&n2, &level_dom, &evt, &nevt_dev, &nevt, &first, &G, &st};
    return cudaLaunchCooperativeKernel(reinterpret_cast<void*>(k_ac_front<WT, TB>), dim3(grid), dim3(kFrontBlock),
                                       args, 0, s);
  });
}

int sac_blocks_per_sm(const DevNet& N, int block, bool smem_state) {
  const size_t smem = smem_state ? cta_state_bytes(N) : 0;
  int per_sm = 0;
  cudaError_t e = dispatch_wt(N, [&](auto wt, auto tab) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    constexpr bool TB = decltype(tab)::value;
    cudaError_t e2 = allow_smem(k_sac<WT, TB>, smem);
    if (e2 != cudaSuccess) return e2;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sac<WT, TB>, block, smem);
  });
  return e == cudaSuccess ? per_sm : 0;
}

cudaError_t launch_sac_branches(const DevNet& N, const u64* root, const int2* work, const int* nwork, int* cursor,
                                uint8_t* ok, KStats* st, int block, int grid, void* gscratch, size_t gstride,
                                cudaStream_t s, const int* idx, const int* nidx, u64* gs_root) {
  const size_t smem = gscratch ? 0 : cta_state_bytes(N);
  const int* count = idx ? nidx : nwork;
  return dispatch_wt(N, [&](auto wt, auto tab) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    constexpr bool TB = decltype(tab)::value;
    cudaError_t e = allow_smem(k_sac<WT, TB>, smem);
    if (e != cudaSuccess) return e;
    return launch_pdl(k_sac<WT, TB>, dim3(grid), dim3(block), smem, s, N, root, work, count, cursor, ok, st,
                      static_cast<char*>(gscratch), gstride, idx, gs_root);
  });
}

size_t sac_tile_smem(const DevNet& N, int slot_cap) {
  return static_cast<size_t>(slot_cap) * (32 * N.W * 8 + 16) + static_cast<size_t>(N.n) * 4;
}

int sac_tile_blocks_per_sm(const DevNet& N, int slot_cap, int block) {
  const size_t smem = sac_tile_smem(N, slot_cap);
  int per_sm = 0;
  cudaError_t e = dispatch_w(N.W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    cudaError_t e2 = allow_smem(k_sac_tile<WT>, smem);
    if (e2 != cudaSuccess) return e2;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sac_tile<WT>, block, smem);
  });
  return e == cudaSuccess ? per_sm : 0;
}

cudaError_t launch_sac_tile(const DevNet& N, u64* root, SacScratch S, uint8_t* ok, int slot_cap, KStats* st,
                            int block, int grid, cudaStream_t s) {
  if (block > 256 || block % 32) return cudaErrorInvalidValue;  // per-warp shared arrays are sized for 256
  const size_t smem = sac_tile_smem(N, slot_cap);
  return dispatch_w(N.W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    cudaError_t e = allow_smem(k_sac_tile<WT>, smem);
    if (e != cudaSuccess) return e;
    return launch_pdl(k_sac_tile<WT>, dim3(grid), dim3(block), smem, s, N, root, S.snap, S.tiles, S.ntiles,
                      S.tcursor, ok, S.deep, S.ndeep, slot_cap, st, S.weak);
  });
}

cudaError_t launch_work_and_weak(const DevNet& N, const u64* dom, SacScratch S, u64* snap, u32* weak,
                                 cudaStream_t s) {
  return dispatch_w(N.W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    const int wb = std::max(1, std::min(4096, (N.n * 32 + 255) / 256));
    const int kb = std::max(1, std::min(8192, (2 * N.nb * 32 + 255) / 256));
    return launch_pdl(k_work_and_weak<WT>, dim3(wb + kb), dim3(256), 0, s, N, dom, S.work, S.nwork, S.tiles,
                      S.ntiles, snap, weak, wb);
  });
}

cudaError_t launch_build_work(const DevNet& N, const u64* dom, SacScratch S, u64* snap, cudaStream_t s) {
  return dispatch_w(N.W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    const int blocks = std::max(1, std::min(4096, (N.n * 32 + 255) / 256));
    k_build_work<WT><<<blocks, 256, 0, s>>>(N, dom, S.work, S.nwork, S.tiles, S.ntiles, snap);
    return cudaGetLastError();
  });
}

// Start of a SAC round: the round's two stats slots (fail_var -1, the rest
// zero) and, for the grid fixpoint, its control block (flags .. bitmaps).
__global__ void k_round_prep(KStats* st, int* ctl, int ctl_words) {
  constexpr int kw = static_cast<int>(sizeof(KStats) / sizeof(int));
  int* p = reinterpret_cast<int*>(st);
  for (int i = threadIdx.x; i < 2 * kw; i += blockDim.x) p[i] = 0;
  for (int i = threadIdx.x; i < ctl_words; i += blockDim.x) ctl[i] = 0;
  __syncthreads();
  if (threadIdx.x == 0) st[0].fail_var = st[1].fail_var = -1;
}

// After the round's level AC has read the previous commit's events: the sweep
// counters (nwork .. ndeep) and the changed-variable bitmap.
__global__ void k_round_clear(int* ctr, int nctr, u32* fb, int nw) {
  pdl_wait();
  for (int i = threadIdx.x; i < nctr; i += blockDim.x) ctr[i] = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x) fb[i] = 0u;
}

// Copies k stats slots to host-mapped memory, visible to the host once the
// stream has been synchronised.
__global__ void k_stats_out(const KStats* src, KStats* dst, int k) {
  constexpr int kw = static_cast<int>(sizeof(KStats) / sizeof(int));
  const int* a = reinterpret_cast<const int*>(src);
  int* b = reinterpret_cast<int*>(dst);
  for (int i = threadIdx.x; i < k * kw; i += blockDim.x) b[i] = a[i];
  __threadfence_system();
}

cudaError_t launch_stats_out(const KStats* src, KStats* dst, int k, cudaStream_t s) {
  k_stats_out<<<1, 64, 0, s>>>(src, dst, k);
  return cudaGetLastError();
}

cudaError_t launch_round_prep(KStats* st, int* ctl, int ctl_words, cudaStream_t s) {
  k_round_prep<<<1, 256, 0, s>>>(st, ctl, ctl_words);
  return cudaGetLastError();
}

cudaError_t launch_round_clear(int* ctr, int nctr, u32* fb, int nw, cudaStream_t s) {
  const int blocks = std::max(1, std::min(64, (nw + 255) / 256));
  return launch_pdl(k_round_clear, dim3(blocks), dim3(256), 0, s, ctr, nctr, fb, nw);
}

cudaError_t launch_commit(const DevNet& N, u64* dom, SacScratch S, KStats* st, KStats* out, int nst, u64* dom_out,
                          cudaStream_t s) {
  const int blocks = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(4096, (N.total_values + 255) / 256)));
  return launch_pdl(k_commit, dim3(blocks), dim3(256), 0, s, N.W, S.work, S.nwork, S.ok, dom, S.evt, S.nevt,
                    S.evt_fb, st, reinterpret_cast<unsigned*>(S.nwork + 7), out, nst, dom_out,
                    static_cast<size_t>(N.n) * N.W);
}

cudaError_t launch_transpose(const DevNet& N, u64* rel, const int* bx, const int* by, const int64_t* offA,
                             const int64_t* offB, cudaStream_t s) {
  if (N.nb == 0) return cudaSuccess;
  const int chunks = 2 * N.W;  // 32-value groups of y
  return dispatch_w(N.W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    const int64_t warps = static_cast<int64_t>(N.nb) * chunks;
    const int blocks = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(8192, (warps * 32 + 255) / 256)));
    k_transpose<WT><<<blocks, 256, 0, s>>>(N, rel, bx, by, offA, offB, chunks);
    return cudaGetLastError();
  });
}

cudaError_t launch_popcount(const DevNet& N, const u64* dom, int* sizes, cudaStream_t s) {
  return dispatch_w(N.W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    const int blocks = std::max(1, std::min(1024, (N.n + 255) / 256));
    k_popcount<WT><<<blocks, 256, 0, s>>>(N.n, dom, sizes);
    return cudaGetLastError();
  });
}

cudaError_t launch_level_edit(const DevNet& N, u64* dom, int var, int val, int op, cudaStream_t s) {
  k_level_edit<<<1, 1, 0, s>>>(N.W, dom, var, val, op);
  return cudaGetLastError();
}

cudaError_t launch_gen_rows(const DevNet& N, u64* rel, const int* bx, const int* by, const int64_t* offA,
                            const u64* cseed, const u32* thr, cudaStream_t s) {
  if (N.nb == 0) return cudaSuccess;
  const int blocks = std::max(1, std::min(16384, (N.nb * 32 + 255) / 256));
  k_gen_rows<<<blocks, 256, 0, s>>>(N.nb, N.W, N.dsize, rel, bx, by, offA, cseed, thr);
  return cudaGetLastError();
}

// ---- batches ----

int batch_node_blocks_per_sm(int W, bool tables, int block, size_t smem) {
  int per_sm = 0;
  cudaError_t e = dispatch_wtab(W, tables, [&](auto wt, auto tab) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    constexpr bool TB = decltype(tab)::value;
    cudaError_t e2 = allow_smem(k_batch_node<WT, TB>, smem);
    if (e2 != cudaSuccess) return e2;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_node<WT, TB>, block, smem);
  });
  return e == cudaSuccess ? per_sm : 0;
}

cudaError_t launch_batch_node(int W, bool tables, const BatchDev& B, int op, KStats* st, int block, int grid,
                              size_t smem, void* gscratch, size_t gstride, cudaStream_t s) {
  return dispatch_wtab(W, tables, [&](auto wt, auto tab) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    constexpr bool TB = decltype(tab)::value;
    cudaError_t e = allow_smem(k_batch_node<WT, TB>, smem);
    if (e != cudaSuccess) return e;
    k_batch_node<WT, TB><<<grid, block, gscratch ? 0 : smem, s>>>(B, op, st, static_cast<char*>(gscratch), gstride);
    return cudaGetLastError();
  });
}

cudaError_t launch_batch_build(int W, const BatchDev& B, bool with_tiles, cudaStream_t s) {
  return dispatch_w(W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    const int blocks = std::max(1, std::min(8192, (B.total_vars * 32 + 255) / 256));
    k_batch_build<WT><<<blocks, 256, 0, s>>>(B, with_tiles ? 1 : 0);
    return cudaGetLastError();
  });
}

cudaError_t launch_batch_snap(int W, const BatchDev& B, cudaStream_t s) {
  k_batch_snap<<<std::max(1, std::min(B.k, 4096)), 256, 0, s>>>(B, W);
  return cudaGetLastError();
}

cudaError_t launch_batch_weak(int W, const BatchDev& B, cudaStream_t s) {
  return dispatch_w(W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    const int blocks = std::max(1, std::min(8192, (B.total_vars * 32 + 255) / 256));
    k_batch_weak<WT><<<blocks, 256, 0, s>>>(B);
    return cudaGetLastError();
  });
}

size_t batch_tile_smem(int W, int slot_cap, int max_n) {
  return static_cast<size_t>(slot_cap) * (32 * W * 8 + 16) + static_cast<size_t>(max_n) * 4;
}

int batch_tile_blocks_per_sm(int W, int slot_cap, int max_n) {
  const size_t smem = batch_tile_smem(W, slot_cap, max_n);
  int per_sm = 0;
  cudaError_t e = dispatch_w(W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    cudaError_t e2 = allow_smem(k_batch_tile<WT>, smem);
    if (e2 != cudaSuccess) return e2;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_tile<WT>, 256, smem);
  });
  return e == cudaSuccess ? per_sm : 0;
}

cudaError_t launch_batch_tile(int W, const BatchDev& B, int slot_cap, int max_n, KStats* st, int grid, int quota,
                              cudaStream_t s) {
  const size_t smem = batch_tile_smem(W, slot_cap, max_n);
  return dispatch_w(W, [&](auto wt) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    cudaError_t e = allow_smem(k_batch_tile<WT>, smem);
    if (e != cudaSuccess) return e;
    k_batch_tile<WT><<<grid, 256, smem, s>>>(B, slot_cap, max_n, st, quota);
    return cudaGetLastError();
  });
}

int batch_sac_blocks_per_sm(int W, bool tables, int block, size_t smem) {
  int per_sm = 0;
  cudaError_t e = dispatch_wtab(W, tables, [&](auto wt, auto tab) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    constexpr bool TB = decltype(tab)::value;
    cudaError_t e2 = allow_smem(k_batch_sac<WT, TB>, smem);
    if (e2 != cudaSuccess) return e2;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_sac<WT, TB>, block, smem);
  });
  return e == cudaSuccess ? per_sm : 0;
}

cudaError_t launch_batch_sac(int W, bool tables, const BatchDev& B, bool deep_only, KStats* st, int block, int grid,
                             size_t smem, void* gscratch, size_t gstride, int quota, cudaStream_t s) {
  return dispatch_wtab(W, tables, [&](auto wt, auto tab) -> cudaError_t {
    constexpr int WT = decltype(wt)::value;
    constexpr bool TB = decltype(tab)::value;
    cudaError_t e = allow_smem(k_batch_sac<WT, TB>, smem);
    if (e != cudaSuccess) return e;
    k_batch_sac<WT, TB><<<grid, block, gscratch ? 0 : smem, s>>>(B, deep_only ? 1 : 0, st,
                                                                 static_cast<char*>(gscratch), gstride, quota);
    return cudaGetLastError();
  });
}

cudaError_t launch_batch_commit(int W, const BatchDev& B, KStats* st, cudaStream_t s) {
  k_batch_commit<<<2048, 256, 0, s>>>(B, W, st);
  return cudaGetLastError();
}

cudaError_t launch_batch_copy(int W, const BatchDev& B, int src_level, cudaStream_t s) {
  k_batch_copy<<<std::max(1, std::min(B.k, 4096)), 256, 0, s>>>(B, W, src_level);
  return cudaGetLastError();
}

cudaError_t launch_batch_edit(int W, const BatchDev& B, int n_edit, const int* member, const int* var, const int* val,
                              cudaStream_t s) {
  if (n_edit <= 0) return cudaSuccess;
  k_batch_edit<<<(n_edit + 255) / 256, 256, 0, s>>>(B, W, n_edit, member, var, val);
  return cudaGetLastError();
}

cudaError_t launch_batch_gather(int W, const BatchDev& B, u64* out, cudaStream_t s) {
  k_batch_gather<<<std::max(1, std::min(B.k, 4096)), 256, 0, s>>>(B, W, out);
  return cudaGetLastError();
}

cudaError_t launch_batch_select(const BatchDev& B, bool initial, cudaStream_t s) {
  const int blocks = std::max(1, std::min(1024, (B.k + 255) / 256));
  k_batch_select<<<blocks, 256, 0, s>>>(B, initial ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace cpgpu
