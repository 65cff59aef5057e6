// Internal layout shared by the host engine (cp_engine.cu) and the kernels
// (cp_kernels.cu). Plain structs of device pointers, passed by value to
// kernels.
//
// HBM layout of one network (all u64 words, W = internal words per domain,
// 1, 2, 4 or 8; a user W of 3 is padded to 4 and 5..8 to 8):
//   levels   [L][n][W]          domain stack, level 0 = root
//   rel      [A blocks][B blocks]
//            A block of binary constraint c = (x, y): dom[x] rows of W words,
//            row a = supports of x=a among y's values (the user's rows);
//            B block: dom[y] rows, row b = supports of y=b among x's values
//            (the transpose, built on the device at upload).
//   arcs     grouped by source variable y: revising z against y for every
//            constraint linking y and z; zy = word offset of z's rows (bits
//            over y), yz = offset of y's rows (bits over z).
//   tables   u16 tuples, column-major per table (coordinate i of all tuples
//            contiguous) for coalesced loads; incidence var -> tables.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace cpgpu {

using u64 = unsigned long long;
using u32 = unsigned int;

// Tables up to this arity (and at most 256 values per domain) are revised with
// every scope position's domain and projection in registers; wider ones a few
// positions at a time.
constexpr int kMaxArity = 4;
// Lanes that revise one binary arc together in the CTA fixpoints, by domain
// words: each lane tests at most 8 values per pass, so a warp revises 4 arcs
// at once for domains of up to 64 values and 2 for up to 128; wider domains
// take the whole warp per arc.
__host__ __device__ constexpr int arc_group_lanes(int W) { return W == 1 ? 8 : W == 2 ? 16 : 32; }
// Weak-support lists of the tiled SAC sweep: per directional arc, kWeakStride
// words (80 bytes, 16-byte aligned): the support count of the (kWeakK+1)-th
// weakest value, then the kWeakK values of the revised variable with the
// fewest supports, then padding.
constexpr int kWeakK = 16;
constexpr int kWeakStride = 20;
constexpr int kMaxVars = 1 << 20;             // variables per network

struct Arc {
  int z;        // variable revised
  u32 zy;       // word offset of z's rows (value-wise revise)
  u32 yz;       // word offset of y's rows (union-of-supports revise)
  int src;      // y, the variable whose incidence list holds the arc
};

struct DevNet {
  int n = 0, W = 1, nb = 0, nt = 0;
  int chunk = 8;          // incidences per work item
  int64_t total_values = 0;
  const int* dsize = nullptr;       // [n]
  const int* arc_start = nullptr;   // [n+1]
  const Arc* arcs = nullptr;        // [2*nb]
  const int* tinc_start = nullptr;  // [n+1]
  const int* vtab = nullptr;        // table ids per variable
  const u64* rel = nullptr;
  const int* t_arity = nullptr;
  const int* t_scope = nullptr;     // scopes of all tables, concatenated
  const int* t_soff = nullptr;      // [nt] start of table t's scope in t_scope
  const int* t_scope4 = nullptr;    // [nt * kMaxArity] the first kMaxArity scope positions at a fixed stride
  const int* t_ntup = nullptr;
  const int64_t* t_off = nullptr;   // offset of table t's tuples in t_tup
  const uint16_t* t_tup = nullptr;
};

// Counters of one propagation call, accumulated on the device.
struct KStats {
  u64 revisions;
  u64 rows;           // binary support rows read
  u64 tuples;         // table tuples scanned
  u64 deletions;
  u64 fixpoints;
  u64 branches;
  u64 removed;        // SAC: values removed by failed singleton tests
  int rounds_max;
  int inconsistent;
  int fail_var;
  int error;          // 0, or a CP_E_* code set by a device-side check
  int grid_err;       // bounded grid barrier timeout
  int pad[3];
};

// Global-memory state of the grid-wide fixpoint (one per network): one block
// of ctl_words ints cleared by one memset before each launch.
struct GridScratch {
  int* flags;         // [3] bitmap i has a bit set
  int* failed;        // [2] wipe-out seen, by round parity
  unsigned* bar;      // [2] grid barrier: count, generation
  u32* bm;            // [3][ceil(n/32)] frontier bitmaps
  size_t ctl_words;   // size of the block starting at flags
  long long wait_ns;  // longest wait of a block at the grid barrier
};

// SAC sweep buffers (one per network).
struct SacScratch {
  int2* work;         // live (x, a) pairs, up to total_values
  int* nwork;         // [1]
  uint8_t* ok;        // per pair: singleton test result
  int* cursor;        // [1] next branch for the persistent CTAs
  int* evt;           // variables changed by a commit, up to n
  int* nevt;          // [1]
  u32* evt_fb;        // dedupe bitmap for evt
  int4* tiles;        // (x, first value, first work index, live mask) per 32 values
  int* ntiles;        // [1]
  int* tcursor;       // [1]
  int* deep;          // work indices the tiled kernel hands to the general one
  int* ndeep;         // [1]
  u32* weak;          // [2*nb][kWeakStride] weak-support lists (null: not built)
  u64* snap;          // [n*W] the level's domains at the start of the sweep
};

enum NodeOp { kOpRoot = 0, kOpAssign = 1, kOpRefute = 2, kOpSingleton = 3, kOpEvents = 4 };

// One device-resident MAC search (k_mac): the whole depth-first search of one
// network runs in one CTA.
// Where a search stands between launches: searches run in time slices, and
// a slice that ends mid-search leaves its state here for the next launch.
struct MacState {
  int phase;             // 0 not started, 1 suspended, 2 finished
  int p, top;            // path depth, highest level with live flags
  int pad;
  long long npos, nneg, props, t_start;
};

struct MacJob {
  MacState* state;       // device memory, zeroed before the first launch
  int net;               // index into the launch's network array
  int levels;            // depth of the level stack
  int varh;              // MAC order 1: dom/min, 0: lex, 4: dom/deg; 2: the d-way search of GModelSolver
  const int* nbr;        // n neighbour counts (dom/deg), else null
  int n_choice;
  const u64* init;       // n*W words: domains before the choices
  u64* stack_dom;        // levels * n * W words
  uint8_t* assigned;     // levels * n flags
  int2* path;            // n + 1 decisions (variable, value)
  const int2* choices;   // n_choice (variable, value): D(var) reduced to {value} before the root
  int* solution;         // n values (host-visible memory)
  long long limit_ns;    // time limit from the start of the job (0: none)
};

// Result of one k_mac job, in host-visible memory; `done` is written last.
struct MacOut {
  int status;            // 1 solution, 0 unsatisfiable, 2 time limit, < 0 error code
  int done;
  long long npos, nneg, props;
};

// A multi-instance batch: networks of one internal domain width, processed
// together by one launch per phase. Work pairs and tiles carry the instance in
// the high 16 bits of their variable field (instance < 32768, n < 65536).
struct BatchDev {
  int k = 0;                     // instances
  int total_vars = 0;            // sum of n over instances
  const DevNet* nets = nullptr;  // [k]
  u64* const* roots = nullptr;   // [k] level each instance works on
  u64* const* bases = nullptr;   // [k] level 0 of each instance's level stack
  const int64_t* out_off = nullptr;  // [k] word offset of the instance in a gathered domain buffer
  const int* wuser = nullptr;    // [k] caller's words per domain (<= W)
  const int* var_base = nullptr; // [k+1] global id of each instance's variable 0
  const int* var_inst = nullptr; // [total_vars] instance of each global variable
  uint8_t* inc = nullptr;        // [k] 1 once known inconsistent
  uint8_t* act = nullptr;        // [k] takes part in the current sweep
  int* removed = nullptr;        // [k] values removed by the last commit
  int* evt = nullptr;            // [total_vars] changed variables, instance i at var_base[i]
  int* nevt = nullptr;           // [k]
  u32* evt_fb = nullptr;         // bitmap over global variables
  int* act_list = nullptr;       // [k] instances for the node kernel
  int* nact = nullptr;           // [1]
  int2* work = nullptr;          // {inst << 16 | x, a}
  int* nwork = nullptr;
  uint8_t* ok = nullptr;
  int* cursor = nullptr;
  int4* tiles = nullptr;         // {inst << 16 | x, first value, first work index, live mask}
  int* ntiles = nullptr;
  int* tcursor = nullptr;
  int* deep = nullptr;
  int* ndeep = nullptr;
  u32* weak = nullptr;             // weak-support lists of all members (null: none)
  u64* snap = nullptr;             // [total_vars*W] members' domains at the sweep start (null: no early removal)
  const int64_t* weak_off = nullptr;  // [k] first list word of each member
};

// Batch launch wrappers (cp_kernels.cu). W / tables select the template.
cudaError_t launch_batch_node(int W, bool tables, const BatchDev& B, int op, KStats* st, int block, int grid,
                              size_t smem, void* gscratch, size_t gstride, cudaStream_t s);
int batch_node_blocks_per_sm(int W, bool tables, int block, size_t smem);
cudaError_t launch_batch_build(int W, const BatchDev& B, bool with_tiles, cudaStream_t s);
cudaError_t launch_batch_tile(int W, const BatchDev& B, int slot_cap, int max_n, KStats* st, int grid, int quota,
                              cudaStream_t s);
size_t batch_tile_smem(int W, int slot_cap, int max_n);
int batch_tile_blocks_per_sm(int W, int slot_cap, int max_n);
cudaError_t launch_batch_sac(int W, bool tables, const BatchDev& B, bool deep_only, KStats* st, int block, int grid,
                             size_t smem, void* gscratch, size_t gstride, int quota, cudaStream_t s);
int batch_sac_blocks_per_sm(int W, bool tables, int block, size_t smem);
cudaError_t launch_batch_commit(int W, const BatchDev& B, KStats* st, cudaStream_t s);
cudaError_t launch_batch_select(const BatchDev& B, bool initial, cudaStream_t s);
// Copies level (batch level + delta) onto the batch level for every member.
cudaError_t launch_batch_copy(int W, const BatchDev& B, int src_level, cudaStream_t s);
cudaError_t launch_batch_weak(int W, const BatchDev& B, cudaStream_t s);
// MAC searches (any widths and network kinds in one launch); CTA state in
// shared memory (smem bytes) or per-CTA global scratch (gscratch, gstride).
cudaError_t launch_mac(const DevNet* nets, const MacJob* jobs, int njobs, int* cursor, MacOut* outs, int block,
                       int grid, size_t smem, void* gscratch, size_t gstride, long long slice_ns, cudaStream_t s);
int mac_blocks_per_sm(int block, size_t smem);
cudaError_t launch_batch_edit(int W, const BatchDev& B, int n_edit, const int* member, const int* var, const int* val,
                              cudaStream_t s);
cudaError_t launch_batch_gather(int W, const BatchDev& B, u64* out, cudaStream_t s);

// Shared-memory (or per-CTA scratch) bytes of the CTA-local fixpoint.
size_t cta_state_bytes(const DevNet& N);

// ---- launch wrappers (cp_kernels.cu) ----
// One CTA: domains of level src loaded to the CTA's state, the operation
// applied, fixpoint computed, result written to level dst (unless singleton).
cudaError_t launch_node(const DevNet& N, u64* levels, int src, int dst, int op, int var, int val,
                        const int* evt, int nevt, KStats* st, uint8_t* ok_out, int block, void* gscratch,
                        cudaStream_t s);
// Grid-wide fixpoint at level `level`, seeded with evt (or all variables when
// evt == nullptr), the frontier kept in bitmaps (k_ac_front); the GridScratch
// block must be zero on entry. Without evt, round 0 is a plain launch before
// the cooperative one (two launches). ac_front_blocks: the cooperative grid
// for a network with narcs binary incidences (0 if the kernel does not fit).
cudaError_t launch_ac_front(const DevNet& N, u64* level_dom, const int* evt, const int* nevt_dev, int nevt,
                            GridScratch G, KStats* st, int grid, cudaStream_t s);
int ac_front_blocks(const DevNet& N, int narcs, int sm_count);
// Scratch of the sequential AC3 replay (dom/wdeg weights).
struct ReplayScratch {
  unsigned long long* stamp_var;  // [n]
  unsigned long long* stamp_tab;  // [nb]
  int* q;                         // [n + 1] ring
  uint8_t* inq;                   // [n]
};
// The constraint whose revision first empties a domain when AC3 runs in the
// reference's sequential order on D (the node's domains before the edit
// op/var/val; overwritten) with the level's assigned flags: out[0], -1 if
// none. One warp.
cudaError_t launch_ac3_replay(const DevNet& N, const int* arc_con, const int* bx, const int* by, u64* D,
                              const uint8_t* assigned, int op, int var, int val, ReplayScratch R, int* out,
                              cudaStream_t s);
// One SAC support-count tile (cp_tensor.cu): branches x = a for a < dx, rows of
// x over y at word offset xy; values of z (dz of them) with rows over y at zy.
struct SacTile {
  u32 xy, zy;
  int y, z, dx, dz, pad0, pad1;
};
// out[t][a] (two words): values of z in D(z) that lose every support in
// D(y) & row_xy(a); W (internal words per domain) 1 or 2.
cudaError_t launch_tiles_bitwise(int W, const u64* rel, const u64* dom, const SacTile* tiles, int ntiles, u64* out,
                                 int sm_count, cudaStream_t s);
// The same on the tensor cores; *err set to 1 if a product did not complete
// within the bounded wait.
cudaError_t launch_tiles_tc(int W, const u64* rel, const u64* dom, const SacTile* tiles, int ntiles, u64* out,
                            int* err, int sm_count, cudaStream_t s);
// Persistent batched singleton tests: pairs work[0..*nwork), results in ok.
// With idx != nullptr the tests are work[idx[i]] for i < *nidx.
cudaError_t launch_sac_branches(const DevNet& N, const u64* root, const int2* work, const int* nwork, int* cursor,
                                uint8_t* ok, KStats* st, int block, int grid, void* gscratch, size_t gstride,
                                cudaStream_t s, const int* idx = nullptr, const int* nidx = nullptr,
                                u64* gs_root = nullptr);
int sac_blocks_per_sm(const DevNet& N, int block, bool smem_state);
// Tiled singleton tests (binary networks): 32 branches of one variable per
// tile; branches that need more than two propagation rounds are appended to
// S.deep for the general kernel. slot_cap: neighbours held in shared memory.
cudaError_t launch_sac_tile(const DevNet& N, u64* root, SacScratch S, uint8_t* ok, int slot_cap, KStats* st,
                            int block, int grid, cudaStream_t s);
cudaError_t launch_batch_snap(int W, const BatchDev& B, cudaStream_t s);
// Weak-support lists of every arc for the domains at root (into S.weak).
size_t sac_tile_smem(const DevNet& N, int slot_cap);
int sac_tile_blocks_per_sm(const DevNet& N, int slot_cap, int block);
// Builds the list of live (x, a) pairs of a level (warp ballot + prefix);
// when S.tiles is set, also one tile per 32-value slice with live values.
cudaError_t launch_build_work(const DevNet& N, const u64* dom, SacScratch S, u64* snap, cudaStream_t s);
cudaError_t launch_work_and_weak(const DevNet& N, const u64* dom, SacScratch S, u64* snap, u32* weak,
                                 cudaStream_t s);
cudaError_t launch_round_prep(KStats* st, int* ctl, int ctl_words, cudaStream_t s);
cudaError_t launch_stats_out(const KStats* src, KStats* dst, int k, cudaStream_t s);
cudaError_t launch_round_clear(int* ctr, int nctr, u32* fb, int nw, cudaStream_t s);
// Removes failed pairs from the level, collecting changed variables.
// out (host-mapped, may be null): the last block copies nst stats slots there
// and, with dom_out (host-mapped, may be null) and no removal in the sweep,
// the level's n * W words; S.nwork + 7 is its completion counter (zero
// between launches).
cudaError_t launch_commit(const DevNet& N, u64* dom, SacScratch S, KStats* st, KStats* out, int nst, u64* dom_out,
                          cudaStream_t s);
// Builds the B blocks (transposes) of the binary relations.
cudaError_t launch_transpose(const DevNet& N, u64* rel, const int* bx, const int* by, const int64_t* offA,
                             const int64_t* offB, cudaStream_t s);
// Fills the A blocks of seeded random relations on the device (cp_gen.h's
// relation_word, the same bits as the host generator).
cudaError_t launch_gen_rows(const DevNet& N, u64* rel, const int* bx, const int* by, const int64_t* offA,
                            const u64* cseed, const u32* thr, cudaStream_t s);
// Sets the message returned by cp_last_error_string on this thread.
void set_last_error(const std::string& msg);
// Level helpers.
cudaError_t launch_popcount(const DevNet& N, const u64* dom, int* sizes, cudaStream_t s);
cudaError_t launch_level_edit(const DevNet& N, u64* dom, int var, int val, int op, cudaStream_t s);

}  // namespace cpgpu
