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
 *   - table t has arity tab_arity[t] (2..n, distinct variables), its scope
 *     in tab_scope and tab_ntup[t] tuples of positive (support) semantics in
 *     tab_tuples, arity ints per tuple, both concatenated over t (the
 *     kSupports ExtensionConstraint of include/model/types.h:148-161; any
 *     arity, like the generic table revise of src/AC3.cpp:195-209).
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
  CP_E_STATE = -6,    /* call not valid in the current state */
  CP_E_CANCELLED = -7 /* a server request cancelled before it ran */
};

typedef struct cp_engine cp_engine;
typedef struct cp_net cp_net;
typedef struct cp_instance cp_instance;

/* Result of one propagation call (ConsistencyState of include/Solver.h:84-97
 * and GacStats of include/GModel.cuh:17-21, widened). */
typedef struct cp_stats {
  int32_t inconsistent;  /* 1 if a domain was wiped out (or SAC closure empty) */
  int32_t rounds;        /* frontier rounds of the last fixpoint (max over branches) */
  int64_t deletions;     /* values removed at the target level by this call */
  int64_t revisions;     /* arc / table revisions performed */
  int64_t rows;          /* support rows and tuples read by revisions */
  int64_t fixpoints;     /* AC closures computed (1, or the SAC branches + root ACs) */
  int64_t branches;      /* SAC singleton tests run (scheduling-dependent with early removals) */
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
/* CUDA device index the engine was created on (-1 for a null engine). */
int cp_engine_device(const cp_engine* e);
/* Engine knobs (normally chosen by the autotuner): 0 = automatic.
 * block: threads per CTA; chunk: incidences per work item; ctas_per_sm:
 * resident CTAs per SM for the batched kernels. */
int cp_engine_set_tuning(cp_engine* e, int block, int chunk, int ctas_per_sm);
/* SAC sweep kernel: 0 = tiled (32 branches of one variable per tile, two-round
 * test, deeper branches re-run by the general kernel) wherever the network is
 * binary and fits, 1 = general per-branch kernel only. Results are identical. */
int cp_engine_set_sac_mode(cp_engine* e, int mode);
/* Single-network SAC1 (cp_enforce_sac1): 1 (default) replays each round (level
 * AC + sweep) as a CUDA graph captured on first use per level, 0 launches its
 * operations one by one. Results are identical. */
int cp_engine_set_graphs(cp_engine* e, int use_graphs);
/* Stream priority of the engine (-1 low, 0 default, 1 high); only before the
 * first network is uploaded. CTAs of a high-priority stream are scheduled
 * first whenever SM resources free up. */
int cp_engine_set_priority(cp_engine* e, int priority);
/* Batch sweeps with quota > 0 launch CTAs that each take at most `quota`
 * tiles or branches and retire, instead of persistent CTAs, so that
 * higher-priority work on other streams gets SMs during long sweeps. Results
 * are unchanged. Applies to batches created afterwards. */
int cp_engine_set_cta_quota(cp_engine* e, int quota);
/* Longest wait of a CTA at the grid-wide barrier of the persistent fixpoint
 * kernel (default 2 s); past it the kernel stops and the call returns
 * CP_E_TIMEOUT, leaving the context usable. Failure handling and its tests. */
int cp_engine_set_wait_budget(cp_engine* e, int64_t ns);
/* Test hook: after `after` more device allocations of this engine succeed,
 * the next one fails as out of memory (CP_E_OOM); -1 turns it off. */
int cp_engine_inject_alloc_failure(cp_engine* e, int64_t after);

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
/* The same, returning once the copies (and the device-side derivation of the
 * other relation side) are queued on a lowest-priority transfer stream of
 * the engine that its own stream then waits on: work of other engines
 * proceeds meanwhile (with a higher stream priority, cp_engine_set_priority,
 * it keeps the SMs first), and this network's next call runs after the
 * reload. bin_rows must stay unchanged until that call (pinned memory
 * overlaps the copy with other work). No counterpart in the reference. */
int cp_net_reload_async(cp_net* net, const uint64_t* init, const uint64_t* bin_rows);

/* ---- level stack (Network::NewLevel/BackTo/CopyLevel, src/Network.cpp:438-455;
 *      IntVar::RemoveValue/ReduceTo, :106-118; GModel level API,
 *      include/GModel.cuh:219-253) --------------------------------------- */
int cp_level_copy(cp_net* net, int src, int dst);
int cp_dom_get(cp_net* net, int level, uint64_t* out);      /* n*W words */
int cp_dom_set(cp_net* net, int level, const uint64_t* in); /* n*W words */
int cp_dom_sizes(cp_net* net, int level, int* out);         /* n popcounts */
int cp_reduce_to(cp_net* net, int level, int var, int value);
int cp_remove(cp_net* net, int level, int var, int value);
/* Network::NewLevel(src) (src/Network.cpp:438-442): level src + 1 := level
 * src, which becomes the top; *new_level = src + 1. */
int cp_level_push(cp_net* net, int src, int* new_level);
/* Network::BackTo(p) (src/Network.cpp:444-446, IntVar::BackTo :235-239):
 * level p becomes the top; the data of every level is left as it is. */
int cp_level_pop_to(cp_net* net, int level);
/* The top level set by the last cp_level_push / cp_level_pop_to (0 at upload). */
int cp_level_top(const cp_net* net);
/* The domain of one variable at a level: W words, bits past its size cleared
 * (the per-variable form of cp_dom_set). */
int cp_dom_set_var(cp_net* net, int level, int var, const uint64_t* words);

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
 * test fails. In SAC mode 0 a failed test also removes its value from the
 * level at once, so later tests of the same sweep start without it; the
 * closure is the same (unique), while the number of tests run depends on
 * scheduling. */
int cp_enforce_sac1(cp_net* net, int level, cp_stats* st);
/* cp_enforce_sac1 in two halves: _begin queues the first round (level AC and
 * sweep) and returns; _end waits for it, runs the further sweeps and fills
 * st. Between the two the host is free (e.g. to queue another network's
 * upload), but the engine takes no other call. No counterpart in the
 * reference. */
int cp_enforce_sac1_begin(cp_net* net, int level);
int cp_enforce_sac1_end(cp_net* net, cp_stats* st);
/* _end that also returns the level's final domains (n*W words, as
 * cp_dom_get): the last sweep's commit kernel writes them to host memory, so
 * no separate read-back follows. */
int cp_enforce_sac1_end_domains(cp_net* net, cp_stats* st, uint64_t* domains);
/* Singleton tests of `count` pairs (vars[i], vals[i]) against the domains of
 * `level` without changing them: ok[i] = 1 if the AC fixpoint of the level
 * with vars[i] reduced to vals[i] is consistent. mode 0 = batched persistent
 * launch, mode 1 = one plain single-instance launch per test (the baseline). */
int cp_singletons(cp_net* net, int level, int count, const int* vars, const int* vals, uint8_t* ok,
                  int mode, cp_stats* st);
/* One Jacobi sweep of singleton tests, through the same kernels as the sweeps
 * of cp_enforce_sac1: AC at `level` first (the level keeps that closure),
 * then every live (x, a) tested against the same domains, nothing removed.
 * The sweep of SAC1::one_pass (src/SAC1.cpp:31-55) and of the loop body of
 * SAC1::enforce (:66-100), without their removals inside the sweep.
 * verdict: n*W words; bit (x, a) is set iff a is in D(x) after the AC and
 * the singleton AC fixpoint of x = a is consistent (all zero if the AC wiped
 * a domain out: st->inconsistent = 1). deep (optional): the tests the
 * two-round tiled kernel passed on to the general fixpoint kernel (0 where
 * the tiled kernel does not run). */
int cp_sac_sweep(cp_net* net, int level, uint64_t* verdict, int64_t* deep, cp_stats* st);
/* Support counting of SAC tiles, bitwise or on the tensor cores: the
 * support-count form of a singleton test's round two that the reference only
 * projects (docs/tensor_core_vs_cuda_core_gac.md), measured beside the
 * bitwise form on the same tiles. Tile t is (x, c1, c2): constraint c1 joins
 * x and y, constraint c2 joins y and z. Its 128 branches are x = a for
 * a < dom(x), with D_a(y) = D(y) & R_c1(x = a) at `level`; out (ntiles * 128 * 2
 * words) gets, per tile and branch a, the values v in D(z) with no support in
 * D_a(y) (the AND-then-any of AC3bit::seek_support, src/AC3bit.cpp:29-38),
 * zero for a >= dom(x). mode 0: bitwise (AND and ballot per branch); mode 1:
 * the 0/1 product D_a(y) x R_c2 on the 5th-generation tensor cores (bf16
 * operands, fp32 counts in tensor memory; exact). Both modes give the same
 * words. Binary networks of at most 128 values. ms: kernel time (CUDA events). */
int cp_sac_tiles(cp_net* net, int level, int ntiles, const int* tile_x, const int* tile_c1, const int* tile_c2,
                 int mode, uint64_t* out, double* ms);

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
/* A batch whose member i works on level levels[i] of nets[i]; one network may
 * appear several times at distinct levels (independent queries on one
 * resident network, each on its own level). */
int cp_batch_create_levels(cp_engine* e, int k, cp_net* const* nets, const int* levels, cp_batch** out);
/* Every member's working level := level src_level of its network, then edit j
 * reduces variable var[j] of member member[j] to the value val[j] (an empty
 * domain if val[j] is no longer in it; several edits of one variable
 * intersect). */
int cp_batch_load(cp_batch* b, int src_level, int n_edit, const int* member, const int* var, const int* val);
/* Working domains of all members, concatenated in member order at each
 * member's own word width (n_i * W_i words each), in one device-to-host copy. */
int cp_batch_dom_get(cp_batch* b, uint64_t* out);

/* ---- request server (continuous batching) ----------------------------------
 * Propagate (type 0: AC / GAC), SAC (type 1) and MAC-solve (type 2: dom/min +
 * min value) requests on one GPU. No counterpart in the reference (it has no
 * server); every result equals the same request run alone through the calls
 * above.
 *
 * Networks: registered once (cp_server_register) they stay resident in HBM,
 * level 0 holding the initial domains and levels 1..slots serving as working
 * levels of concurrent requests; or carried by a request (inst) and uploaded
 * for its lifetime. A request may fix variables to values (choices): the
 * working domains start from the initial ones with D(var[j]) reduced to
 * {val[j]} (a value outside the initial domain, or two values for one
 * variable, answers "inconsistent" without touching the device).
 *
 * A scheduler thread admits queued requests in arrival order while their
 * estimated device footprint fits hbm_budget_bytes (resident networks count
 * for as long as they are registered). The propagate and SAC requests
 * admitted together run as one multi-instance batch per type on batch_engine
 * (up to max_batch per tick; batching = 0 runs them one by one, the
 * one-request-per-launch path). Solves run on solver threads, each on its own
 * engine (solve_engine first). Requests that arrive while a batch is on the
 * GPU are admitted as memory and working levels free up. An instance passed
 * to a request must stay alive until its result is released; register copies
 * the instance. */
typedef struct cp_server cp_server;
typedef struct cp_request {
  int32_t type;               /* 0 propagate, 1 SAC, 2 MAC solve */
  int32_t n_choice;
  int64_t net_id;             /* registered network, or 0: use inst */
  const cp_instance* inst;    /* network carried by the request (net_id == 0) */
  const int* choice_var;      /* n_choice variables ... */
  const int* choice_val;      /* ... fixed to these values */
} cp_request;
typedef struct cp_result {
  int32_t status;        /* 0 queued, 1 running, 2 done, < 0 error code */
  int32_t inconsistent;
  int64_t deletions;     /* values removed from the initial domains (consistent results) */
  int64_t num_positive;  /* MAC solves */
  int64_t num_negative;
  int32_t mac_status;    /* 1 solution, 0 unsatisfiable, 2 time out */
  int32_t type;
  double queue_ms;       /* submit to admission */
  double latency_ms;     /* submit to completion */
} cp_result;
int cp_server_create(cp_engine* batch_engine, cp_engine* solve_engine, int64_t hbm_budget_bytes, int max_batch,
                     int batching, cp_server** out);
int cp_server_destroy(cp_server* s);
/* Time limit of each MAC solve (default 600000 ms; then mac_status = 2). */
int cp_server_set_solve_limit(cp_server* s, int64_t ms);
/* Runs MAC solves on k threads (default 1), each on its own engine/stream;
 * the count only grows. */
int cp_server_set_solvers(cp_server* s, int k);
/* Uploads a resident network with `slots` working levels; CP_E_OOM if its
 * footprint does not fit the budget next to what is already admitted. */
int cp_server_register(cp_server* s, const cp_instance* inst, int slots, int64_t* net_id);
/* Frees a resident network; CP_E_STATE while requests on it are queued or
 * running. */
int cp_server_unregister(cp_server* s, int64_t net_id);
int cp_submit(cp_server* s, const cp_request* req, int64_t* ticket);
/* cp_submit of {type, no choices, the network inst}. */
int cp_submit_instance(cp_server* s, int type, const cp_instance* inst, int64_t* ticket);
/* Cancels a queued request (its status becomes CP_E_CANCELLED); CP_E_STATE
 * once it has been admitted. */
int cp_cancel(cp_server* s, int64_t ticket);
/* Waits up to timeout_ms for a request; CP_E_TIMEOUT if still running. */
int cp_wait(cp_server* s, int64_t ticket, int64_t timeout_ms, cp_result* res);
/* cp_wait without waiting: 0 with *res filled once the request is done,
 * 1 while it is queued or running. */
int cp_poll(cp_server* s, int64_t ticket, cp_result* res);
/* n*W words of a done propagate / SAC request (unspecified if inconsistent);
 * CP_E_STATE if there are none. */
int cp_result_domains(cp_server* s, int64_t ticket, uint64_t* out);
int cp_result_solution(cp_server* s, int64_t ticket, int* out);      /* n values */
int cp_release(cp_server* s, int64_t ticket);
/* Replays an arrival trace (request i submitted t_arrival_s[i] seconds after
 * the call starts) and waits for all; fills latency_ms[i] and status[i];
 * stats[0..7] = lane batches, batched requests, wall seconds, peak admitted
 * bytes, busy seconds of the propagate lane, the SAC lane and the solvers
 * (summed), MAC solves that hit the time limit. */
int cp_server_run_trace(cp_server* s, int k, const double* t_arrival_s, const cp_request* reqs, double* latency_ms,
                        int32_t* status, double* stats);

/* ---- search: MAC on device-resident domains -------------------------------
 * MAC::enforce (src/MAC.cpp:100-165) with the reference's variable and value
 * heuristics (include/Solver.h:55-66: var 0 = VRH_LEX, 1 = VRH_DOM_MIN,
 * 4 = VRH_DOM_DEG_MIN; value 0 = VLH_MIN); the host keeps the reference's
 * control flow, the level stack and every propagation stay on the device.
 * In the device search, dom/min and dom/deg are one block-wide minimum of
 * (key, variable) over the unassigned variables (dom/deg: integer |D(v)| over
 * the number of distinct neighbour variables, -1 without neighbours).
 * 6 = VRH_DOM_WDEG_MIN (binary networks) runs host-driven: constraint weights
 * start at 1 and rise by one for the constraint whose revision first empties
 * a domain in the reference's sequential AC3 order (src/AC3.cpp:122-128),
 * found by replaying each failing node's propagation in that order on the
 * device; the variable is chosen on the host (src/MAC.cpp:387-408). */
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
/* Search placement: 0 (default) runs the whole search of cp_mac_solve and of
 * cp_gsolver_solve on the device, in one CTA, for networks whose fixpoints run
 * in one CTA (node counts and solutions are those of the host-driven search);
 * 1 drives every node from the host. */
int cp_engine_set_search_mode(cp_engine* e, int mode);
/* Threads per CTA of the device searches (cp_mac_solve, cp_gsolver_solve,
 * cp_mac_batch_*): a multiple of 32 in 32..512, or 0 (default) to choose from
 * the number of searches and the network sizes. Results are identical. */
int cp_engine_set_search_block(cp_engine* e, int block);
/* Many MAC searches in one launch (one CTA per search, CTAs take searches
 * from a queue). Search i runs on nets[i] from its level 0 with the next
 * n_choice[i] (choice_var, choice_val) pairs reduced to single values (n_choice
 * may be NULL), in its own level stack, so one network may appear several
 * times. Networks may live on other engines of the device. The time limit
 * counts from the start of each search. Returns at once. */
typedef struct cp_mac_batch cp_mac_batch;
int cp_mac_batch_start(cp_engine* e, int k, cp_net* const* nets, const int* n_choice, const int* choice_var,
                       const int* choice_val, int var_heuristic, int val_heuristic, int64_t time_limit_ms,
                       cp_mac_batch** out);
/* Non-blocking: done[i] = 1 and res[i] filled for the searches that have
 * ended (results are written by the device into host-mapped memory as each
 * search ends); *n_done = their number. */
int cp_mac_batch_poll(cp_mac_batch* b, uint8_t* done, cp_search_result* res, int* n_done);
/* Blocks until every search has ended; res may be NULL. */
int cp_mac_batch_wait(cp_mac_batch* b, cp_search_result* res);
/* The solution of an ended search i (n_i values; meaningful if status 1). */
int cp_mac_batch_solution(cp_mac_batch* b, int i, int* out);
int cp_mac_batch_destroy(cp_mac_batch* b);
/* GModelSolver::Solve (src/GModelSolver.cu:31-102): d-way search, min-domain
 * variable among those with more than one value, all values in order. */
int cp_gsolver_solve(cp_net* net, int64_t time_limit_ms, cp_search_result* res, int* solution);

/* ---- instance generator (seeded, shared with the tests and benchmarks) --- */
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
