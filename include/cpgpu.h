/* cpgpu: GB300-native bitset-domain constraint propagation (AC_3bit, GAC with
 * positive tables, SAC1) behind a plain C ABI.
 *
 * Every entry point returns 0 on success or a negative CP_E* code; the message
 * of the last failure on the calling thread is cp_last_error_string(). No
 * exception crosses the ABI. Pointers are host pointers unless stated. One
 * engine owns one CUDA stream on one device; calls on one engine must not run
 * concurrently from several host threads (use one engine per thread).
 *
 * Data formats (shared with the reference's CPU layout):
 *   - a domain is W u64 words per variable, value a = bit (a & 63) of word
 *     (a >> 6), LSB first; bits at or beyond the variable's size are zero.
 *     This is the byte image of IntVar::bit_doms_[level]
 *     (include/Network.h:102-108, 189) and of GModel::bitDom's u32 words
 *     (include/GModel.cuh:93-95) on a little-endian host;
 *   - binary constraint c has scope (bin_scope[2c], bin_scope[2c+1]) = (x, y)
 *     and dom[x] support rows of W words, concatenated over c in bin_rows: row
 *     a has bit b set iff (x=a, y=b) is allowed (the rows of AC3bit::bitSup_,
 *     src/AC3bit.cpp:3-27, for the x side; the y side is derived on upload);
 *   - table t has arity tab_arity[t] (2..4), its scope in tab_scope and
 *     tab_ntup[t] tuples of positive (support) semantics in tab_tuples,
 *     arity ints per tuple, both concatenated over t (the kSupports
 *     ExtensionConstraint of include/model/types.h:148-161).
 */
#ifndef CPGPU_H
#define CPGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  CP_OK = 0,
  CP_E_ARG = -1,      /* invalid argument (bad var, value, level, size) */
  CP_E_OOM = -2,      /* device or host allocation failed */
  CP_E_CUDA = -3,     /* CUDA runtime error */
  CP_E_TIMEOUT = -4,  /* a device-side bounded wait ran out (kernel returned) */
  CP_E_UNSUPPORTED = -5,
  CP_E_STATE = -6     /* call not valid in the current state */
};

typedef struct cp_engine cp_engine;
typedef struct cp_net cp_net;

/* Result of one propagation call (ConsistencyState of include/Solver.h:84-97
 * and GacStats of include/GModel.cuh:17-21, widened). */
typedef struct cp_stats {
  int32_t inconsistent;  /* 1 if a domain was wiped out (or SAC closure empty) */
  int32_t rounds;        /* frontier rounds of the last fixpoint (max over branches) */
  int64_t deletions;     /* values removed at the target level by this call */
  int64_t revisions;     /* arc / table revisions performed */
  int64_t rows;          /* support rows and tuples read by revisions */
  int64_t fixpoints;     /* AC closures computed (1, or the SAC branches + root ACs) */
  int64_t branches;      /* SAC singleton tests run */
  int32_t sweeps;        /* SAC sweeps */
  int32_t launches;      /* kernel launches issued by this call */
  double device_ms;      /* device time of the call (CUDA events) */
  double alg_bytes;      /* algorithmic bytes of the call (roofline numerator) */
  double kernel_ms;      /* SAC: device time of the batched singleton kernel alone */
  double kernel_bytes;   /* SAC: algorithmic bytes of that kernel */
} cp_stats;

/* ---- engine ------------------------------------------------------------ */
/* Replaces the implicit device state of GModel (include/GModel.cuh:78-283). */
int cp_engine_create(int device, cp_engine** out);
int cp_engine_destroy(cp_engine* e);
const char* cp_last_error_string(void);
/* Kernel launches issued by this engine so far. */
int64_t cp_engine_launches(const cp_engine* e);
/* Engine knobs (normally chosen by the autotuner): 0 = automatic.
 * block: threads per CTA; chunk: incidences per work item; ctas_per_sm:
 * resident CTAs per SM for the batched kernels. */
int cp_engine_set_tuning(cp_engine* e, int block, int chunk, int ctas_per_sm);
/* SAC sweep kernel: 0 = tiled (32 branches of one variable per tile, two-round
 * test, deeper branches re-run by the general kernel) wherever the network is
 * binary and fits, 1 = general per-branch kernel only. Results are identical. */
int cp_engine_set_sac_mode(cp_engine* e, int mode);

/* ---- networks ------------------------------------------------------------ */
/* Uploads a network; replaces GModelAdapter::Build
 * (src/model/gmodel_adapter.cu:44-312) and the Network constructor
 * (src/Network.cpp:358-411). init: n*W words, copied to level 0.
 * max_levels: depth of the level stack (<= 0: n + 3, as IntVar's bit_doms_,
 * src/Network.cpp:78). */
int cp_net_upload(cp_engine* e, int n, const int* dom, int W, const uint64_t* init, int n_bin,
                  const int* bin_scope, const uint64_t* bin_rows, int n_tab, const int* tab_arity,
                  const int* tab_scope, const int* tab_ntup, const int* tab_tuples, int max_levels,
                  cp_net** out);
int cp_net_destroy(cp_net* net);
/* Device bytes held by the network (relations, level stack, scratch). */
int64_t cp_net_device_bytes(const cp_net* net);
/* Replaces the relation rows of an uploaded network with new host rows of the
 * same shape (a fresh upload of the same instance without reallocation). */
int cp_net_reload(cp_net* net, const uint64_t* init, const uint64_t* bin_rows);

/* ---- level stack (Network::NewLevel/BackTo/CopyLevel, src/Network.cpp:438-455;
 *      IntVar::RemoveValue/ReduceTo, :106-118; GModel level API,
 *      include/GModel.cuh:219-253) --------------------------------------- */
int cp_level_copy(cp_net* net, int src, int dst);
int cp_dom_get(cp_net* net, int level, uint64_t* out);      /* n*W words */
int cp_dom_set(cp_net* net, int level, const uint64_t* in); /* n*W words */
int cp_dom_sizes(cp_net* net, int level, int* out);         /* n popcounts */
int cp_reduce_to(cp_net* net, int level, int var, int value);
int cp_remove(cp_net* net, int level, int var, int value);

/* ---- propagation --------------------------------------------------------- */
/* AC fixpoint at `level` (AC_3bit for binary networks, GAC when tables are
 * present), seeded with the changed variables evt (n_evt = 0 or evt = NULL:
 * all variables). Replaces AC::enforce(x_evt, level) (include/Solver.h:315)
 * and GModel::EnforceGAC / EnforceGAC_Persistent (include/GModel.cuh:191,197).
 * The closure is unique, so the result equals the reference's whenever the
 * network stays consistent; on wipe-out only the verdict is defined. */
int cp_enforce_ac(cp_net* net, int level, int n_evt, const int* evt, cp_stats* st);
/* SAC closure at `level` (SAC1::enforce, src/SAC1.cpp:57-103): every live
 * (x, a) is tested by a singleton AC fixpoint, all tests of a sweep batched
 * in one persistent launch, failed values removed and AC re-run, until no
 * test fails. */
int cp_enforce_sac1(cp_net* net, int level, cp_stats* st);
/* Singleton tests of `count` pairs (vars[i], vals[i]) against the domains of
 * `level` without changing them: ok[i] = 1 if the AC fixpoint of the level
 * with vars[i] reduced to vals[i] is consistent. mode 0 = batched persistent
 * launch, mode 1 = one plain single-instance launch per test (the baseline). */
int cp_singletons(cp_net* net, int level, int count, const int* vars, const int* vals, uint8_t* ok,
                  int mode, cp_stats* st);

/* ---- multi-instance batches ----------------------------------------------
 * Many independent networks (each uploaded with cp_net_upload, of any sizes)
 * propagated together: one launch per phase for all members of the same
 * domain width, the sweep loop replayed from a captured CUDA graph. Works on
 * level `level` of every member. No counterpart in the reference beyond its
 * per-instance AC / SAC1 calls, which it batches. */
typedef struct cp_batch cp_batch;
int cp_batch_create(cp_engine* e, int k, cp_net* const* nets, int level, cp_batch** out);
int cp_batch_destroy(cp_batch* b);
/* Root AC of every member; inconsistent[i] (optional, k bytes) = verdict. */
int cp_batch_ac(cp_batch* b, cp_stats* st, uint8_t* inconsistent);
/* AC then SAC closure of every member. */
int cp_batch_sac1(cp_batch* b, cp_stats* st, uint8_t* inconsistent);
/* 1 (default): replay the sweep from a captured CUDA graph; 0: plain launches. */
int cp_batch_set_graphs(cp_batch* b, int use_graphs);
/* Autotuner: times tiled / general sweeps and CTA sizes per member group and
 * caches the choice on disk ($CPGPU_TUNE_CACHE). */
int cp_batch_tune(cp_batch* b);
/* info[0..7] = groups, W, has tables, members, tiled, CTA size, slot capacity,
 * CTA state in shared memory. */
int cp_batch_info(const cp_batch* b, int group, int* info);
/* Copies level src of every member onto the batch's level (one launch per
 * member group), e.g. to restore pristine domains kept at another level. */
int cp_batch_copy_level(cp_batch* b, int src);

/* ---- search: MAC on device-resident domains -------------------------------
 * MAC::enforce (src/MAC.cpp:100-165) with the reference's variable and value
 * heuristics (include/Solver.h:55-66: var 1 = VRH_DOM_MIN, value 0 =
 * VLH_MIN); the host keeps the reference's control flow, the level stack
 * and every propagation stay on the device. */
typedef struct cp_search_result {
  int32_t status;        /* 1 solution, 0 proved unsatisfiable, 2 time out */
  int32_t pad;
  int64_t num_positive;  /* SearchStatistics::num_positive */
  int64_t num_negative;  /* SearchStatistics::num_negative */
  int64_t propagations;  /* AC calls */
  double solve_ms;
} cp_search_result;
int cp_mac_solve(cp_net* net, int var_heuristic, int val_heuristic, int64_t time_limit_ms,
                 cp_search_result* res, int* solution);
/* GModelSolver::Solve (src/GModelSolver.cu:31-102): d-way search, min-domain
 * variable among those with more than one value, all values in order. */
int cp_gsolver_solve(cp_net* net, int64_t time_limit_ms, cp_search_result* res, int* solution);

/* ---- instance generator (seeded, shared with the tests and benchmarks) --- */
typedef struct cp_instance cp_instance;
int cp_gen_binary(int n, int d, int64_t e, double p_lo, double p_hi, double remove, uint64_t seed,
                  cp_instance** out);
int cp_gen_mixed(int n, int d, int64_t e, double p_lo, double p_hi, int k3, int ntup, double remove,
                 uint64_t seed, cp_instance** out);
int cp_gen_uneven(uint64_t seed, int n_lo, int n_hi, int d_cap, cp_instance** out);
int cp_gen_free(cp_instance* inst);
/* sizes[0..7] = n, W, n_bin, n_tab, bin_rows words, tab_scope ints,
 * tab_tuples ints, fingerprint (as int64). */
int cp_gen_sizes(const cp_instance* inst, int64_t* sizes);
/* Copies the instance into caller buffers sized by cp_gen_sizes. */
int cp_gen_export(const cp_instance* inst, int* dom, uint64_t* init, int* bin_scope, uint64_t* bin_rows,
                  int* tab_arity, int* tab_scope, int* tab_ntup, int* tab_tuples);
/* Uploads an instance directly (no host export). */
int cp_net_upload_instance(cp_engine* e, const cp_instance* inst, int max_levels, cp_net** out);
/* The same seeded networks as cp_gen_binary / cp_gen_uneven, with the
 * relation rows generated on the device (bit-identical), for workloads whose
 * relations are too large to generate on the host quickly. */
int cp_gen_binary_device(cp_engine* e, int n, int d, int64_t ne, double p_lo, double p_hi, double remove,
                         uint64_t seed, int max_levels, cp_net** out);
int cp_gen_uneven_device(cp_engine* e, uint64_t seed, int n_lo, int n_hi, int d_cap, int max_levels, cp_net** out);
/* Copies a network's binary support rows (the upload format) back to the host. */
int cp_net_rows_get(cp_net* net, uint64_t* out);

/* ---- allocation-free AC fixpoint ------------------------------------------
 * No counterpart in the reference. For callers that must not allocate device
 * memory while they run: cudaMalloc/cudaFree synchronise the whole device
 * (a stall for a latency-bound search or serving loop), and a host framework
 * that already owns the device memory budget may not let a plugin allocate.
 * The caller keeps a binary network in its own device buffers, in the upload
 * format above: d_dom_size[n], d_bin_scope[2*n_bin], d_bin_rows (dom[x]*W
 * words per constraint), and the domains d_dom[n*W] (level image, updated in
 * place to the AC fixpoint; bits beyond each size are cleared). On the given
 * stream (NULL = default stream) the call writes d_status[0..3] =
 * {inconsistent, deletions, rounds, error code}. It calls no cudaMalloc,
 * cudaFree or allocating library routine: all scratch is one static device
 * array of 9 MiB in the library, held on every GPU that loads it until exit.
 * Limits: n <= 2048, W <= 2 (128 values), n_bin <= 2048; larger sizes return
 * CP_E_ARG. All calls on a device share that array (each clears what must
 * start at zero); calls that overlap on the GPU race. The first call on a
 * device sets up the array's device address, so make it before any stream
 * capture. */
int cp_enforce_ac_static(int n, int W, const int* d_dom_size, uint64_t* d_dom, int n_bin, const int* d_bin_scope,
                         const uint64_t* d_bin_rows, int64_t* d_status, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CPGPU_H */
