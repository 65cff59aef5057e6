/* CPU oracle for bitset-domain propagation. TEST INFRASTRUCTURE ONLY: it is the
 * checker for the GPU engine and must never be linked into, or called by, the
 * product library. Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference legs may load it.
 *
 * Each function restates the reference algorithm it names (file:line of
 * leezear2022/cpim). Parity is pinned against the reference itself: the
 * reference sources are compiled unmodified by oracle/ref/Makefile and their
 * outputs are stored as golden fixtures in tests/golden/ (see
 * tests/golden/make_golden.py), which the CPU test suite checks this oracle
 * against.
 *
 * Network view: n variables, W u64 words per domain, domain sizes dom[n].
 * Binary constraint c has scope (bx[c], by[c]) and dom[bx[c]] support rows of W
 * words, concatenated in constraint order in brows (row a, bit b set iff
 * (x=a, y=b) is allowed). Table t has arity tarity[t], scope and tuples
 * concatenated in tscope / ttup (tntup[t] tuples). Constraint ids are binary
 * constraints first (0..nb-1), then tables (nb..nb+nt-1), the order the
 * reference Network sees them in when the model is built that way.
 * Domains are n*W u64 words, value a = bit (a&63) of word (a>>6).
 */
#ifndef CP_ORACLE_H
#define CP_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrcNet {
  int n, W;
  const int* dom;
  int nb;
  const int* bx;
  const int* by;
  const uint64_t* brows;
  int nt;
  const int* tarity;
  const int* tscope;
  const int* tntup;
  const int* ttup;
} OrcNet;

/* Returns 1 if consistent (dom updated to the fixpoint), 0 on wipe-out. */
int orc_ac3bit(const OrcNet* net, uint64_t* dom, int64_t* deletions);
int orc_gac(const OrcNet* net, uint64_t* dom, int64_t* deletions);
int orc_gac_definitional(const OrcNet* net, uint64_t* dom);
int orc_sac1(const OrcNet* net, uint64_t* dom, int64_t* deletions);
/* status: 1 solution, 0 proved unsat, 2 time out. */
int orc_mac(const OrcNet* net, const uint64_t* dom0, int64_t time_limit_ms, int64_t* num_positive,
            int64_t* num_negative, int* solution);
/* The same with variable heuristic varh: 1 = VRH_DOM_MIN, 4 = VRH_DOM_DEG_MIN,
 * 6 = VRH_DOM_WDEG_MIN (binary networks) (-1 for any other). */
int orc_mac_h(const OrcNet* net, const uint64_t* dom0, int64_t time_limit_ms, int varh, int64_t* num_positive,
              int64_t* num_negative, int* solution);
/* The d-way search of GModelSolver (smallest domain above one value first,
 * every value in order, one GAC fixpoint per child) to the first solution.
 * status: 1 solution, 0 proved unsat, 2 time out. */
int orc_dway(const OrcNet* net, const uint64_t* dom0, int64_t time_limit_ms, int64_t* num_positive,
             int64_t* num_negative, int* solution);
/* Brute force: 1 if a solution exists, 0 if none, -1 if the space exceeds limit. */
int orc_brute_solve(const OrcNet* net, const uint64_t* dom0, double limit);
/* 1 if the full assignment satisfies every constraint. */
int orc_check_solution(const OrcNet* net, const int* solution);
/* Singleton test of (x, a) against dom (unchanged): 1 consistent, 0 wipe-out. */
int orc_singleton(const OrcNet* net, const uint64_t* dom, int x, int a);
/* Runs the singleton tests of `count` live (x, a) pairs, taken evenly spread
 * over all live pairs, on `threads` host threads; returns seconds and the
 * number of failed tests. */
double orc_time_singletons(const OrcNet* net, const uint64_t* dom, int64_t count, int threads,
                           int64_t* failed, int64_t* done);
/* Every live (x, a) of dom (unchanged) tested by the singleton test above,
 * spread over `threads` host threads: verdict (n*W words) gets bit (x, a) set
 * iff a is in D(x) and the test is consistent. Returns the number of failed
 * tests. */
int64_t orc_singleton_verdicts(const OrcNet* net, const uint64_t* dom, int threads, uint64_t* verdict);
/* The SAC closure by Jacobi sweeps on `threads` host threads: AC, then all
 * singleton tests against the same domains, the failed values removed and AC
 * re-run, until a sweep fails nothing. The SAC closure is unique, so dom ends
 * where orc_sac1 (the reference's sequential order) ends. Returns 1 if
 * consistent, 0 on wipe-out; sweeps (optional) counts the sweeps run. */
int orc_sac_jacobi(const OrcNet* net, uint64_t* dom, int threads, int64_t* deletions, int* sweeps);
/* Root AC (AC3bit, or GAC when tables are present) timed `reps` times on
 * fresh copies; returns the best seconds. */
double orc_time_ac(const OrcNet* net, const uint64_t* dom, int reps, int64_t* deletions);

/* Instance generator (cpim_gb300/csrc/cp_gen.h) exposed for CPU-only tests. */
void* orc_gen_binary(int n, int d, int64_t e, double p_lo, double p_hi, double remove, uint64_t seed);
void* orc_gen_mixed(int n, int d, int64_t e, double p_lo, double p_hi, int k3, int ntup, double remove,
                    uint64_t seed);
void* orc_gen_uneven(uint64_t seed, int n_lo, int n_hi, int d_cap);
void orc_gen_free(void* inst);
/* Fills the view with pointers into the instance (valid until freed) and
 * returns the initial domains pointer. */
const uint64_t* orc_gen_view(void* inst, OrcNet* out, uint64_t* fingerprint, int64_t* brows_words,
                             int64_t* ttup_ints, int64_t* tscope_ints);

#ifdef __cplusplus
}
#endif
#endif
