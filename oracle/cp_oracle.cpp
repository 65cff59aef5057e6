// CPU oracle for bitset-domain propagation: TEST INFRASTRUCTURE ONLY (see
// cp_oracle.h). Every routine below restates a reference routine of
// leezear2022/cpim in this project's own code; the citation is given on each.
// Nothing here may be linked into the product library.
#include "cp_oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "cp_gen.h"

namespace {

using u64 = uint64_t;

struct Net {
  int n = 0, W = 1, nb = 0, nt = 0, nc = 0;
  std::vector<int> dom;
  std::vector<int> arity;
  std::vector<std::vector<int>> scope;
  // Binary supports per constraint and scope position: rows for each value of
  // scope[pos], W words each, holding the supports among the other variable.
  std::vector<std::vector<u64>> bsup[2];
  std::vector<const int*> tup;
  std::vector<int> ntup;
  std::vector<std::vector<int>> subs;  // variable -> constraint ids, ascending
};

Net build_net(const OrcNet* v) {
  Net N;
  N.n = v->n;
  N.W = v->W;
  N.nb = v->nb;
  N.nt = v->nt;
  N.nc = v->nb + v->nt;
  N.dom.assign(v->dom, v->dom + v->n);
  N.arity.resize(N.nc);
  N.scope.resize(N.nc);
  N.bsup[0].resize(N.nb);
  N.bsup[1].resize(N.nb);
  N.tup.assign(N.nc, nullptr);
  N.ntup.assign(N.nc, 0);
  int64_t off = 0;
  for (int c = 0; c < N.nb; ++c) {
    const int x = v->bx[c], y = v->by[c];
    N.arity[c] = 2;
    N.scope[c] = {x, y};
    auto& s0 = N.bsup[0][c];
    auto& s1 = N.bsup[1][c];
    s0.assign(v->brows + off, v->brows + off + int64_t(N.dom[x]) * N.W);
    s1.assign(size_t(N.dom[y]) * N.W, 0);
    for (int a = 0; a < N.dom[x]; ++a)
      for (int b = 0; b < N.dom[y]; ++b)
        if ((s0[size_t(a) * N.W + (b >> 6)] >> (b & 63)) & 1ull) s1[size_t(b) * N.W + (a >> 6)] |= 1ull << (a & 63);
    off += int64_t(N.dom[x]) * N.W;
  }
  int64_t so = 0, to = 0;
  for (int t = 0; t < N.nt; ++t) {
    const int c = N.nb + t, r = v->tarity[t];
    N.arity[c] = r;
    N.scope[c].assign(v->tscope + so, v->tscope + so + r);
    N.tup[c] = v->ttup + to;
    N.ntup[c] = v->tntup[t];
    so += r;
    to += int64_t(r) * v->tntup[t];
  }
  // Subscription: for each constraint in order, each scope variable
  // (src/Network.cpp:402-403).
  N.subs.resize(N.n);
  for (int c = 0; c < N.nc; ++c)
    for (int x : N.scope[c]) N.subs[x].push_back(c);
  return N;
}

inline bool have(const u64* D, int W, int x, int a) { return (D[size_t(x) * W + (a >> 6)] >> (a & 63)) & 1ull; }
inline void del_bit(u64* D, int W, int x, int a) { D[size_t(x) * W + (a >> 6)] &= ~(1ull << (a & 63)); }
inline int dsize(const u64* D, int W, int x) {
  int s = 0;
  for (int w = 0; w < W; ++w) s += __builtin_popcountll(D[size_t(x) * W + w]);
  return s;
}
inline int head(const u64* D, int W, int x) {
  for (int w = 0; w < W; ++w) {
    const u64 v = D[size_t(x) * W + w];
    if (v) return w * 64 + __builtin_ctzll(v);
  }
  return -1;
}
inline void reduce_to(u64* D, int W, int x, int a) {
  for (int w = 0; w < W; ++w) D[size_t(x) * W + w] = 0;
  D[size_t(x) * W + (a >> 6)] = 1ull << (a & 63);
}
inline int pos_in_scope(const Net& N, int c, int x) {
  // Tabular::index scans from the end (src/Network.cpp:337-341).
  for (int i = N.arity[c] - 1; i >= 0; --i)
    if (N.scope[c][i] == x) return i;
  return -1;
}

// ---------------------------------------------------------------------------
// AC3 with AC3bit supports: restates AC3::enforce (src/AC3.cpp:127-169),
// AC3::revise (src/AC3.cpp:207-221), AC3bit::seek_support
// (src/AC3bit.cpp:29-38) and the FIFO var_que (src/Solver.cpp:180-214).
// Binary networks only, as AC3bit (src/AC3bit.cpp:3-6).
// ---------------------------------------------------------------------------
struct AC3bit {
  const Net& N;
  std::vector<u64> stamp_var, stamp_tab;
  std::vector<int> q;
  std::vector<char> inq;
  size_t qh = 0, qt = 0;
  u64 t = 0;
  int64_t num_delete = 0;
  int fail_c = -1;  // the constraint whose revision emptied a domain (cs.tab)
  explicit AC3bit(const Net& net) : N(net), stamp_var(net.n), stamp_tab(net.nc), q(net.n + 1), inq(net.n) {}

  void insert(int v) {
    if (!inq[v]) {
      q[qt] = v;
      qt = (qt + 1) % q.size();
      inq[v] = 1;
    }
    ++t;
    stamp_var[v] = t;
  }
  int pop() {
    const int v = q[qh];
    qh = (qh + 1) % q.size();
    inq[v] = 0;
    return v;
  }
  bool seek_support(u64* D, int c, int ypos, int a) const {
    const int z = N.scope[c][1 - ypos];
    const u64* row = &N.bsup[ypos][c][size_t(a) * N.W];
    for (int w = 0; w < N.W; ++w)
      if (row[w] & D[size_t(z) * N.W + w]) return true;
    return false;
  }
  bool revise(u64* D, int c, int y) {
    const int before = dsize(D, N.W, y);
    const int ypos = pos_in_scope(N, c, y);
    for (int a = 0; a < N.dom[y]; ++a) {
      if (!have(D, N.W, y, a)) continue;
      if (!seek_support(D, c, ypos, a)) {
        del_bit(D, N.W, y, a);
        ++num_delete;
      }
    }
    return before != dsize(D, N.W, y);
  }
  // assigned: per-variable flags of the level (nullptr = none assigned).
  bool enforce(u64* D, const std::vector<int>& evt, const char* assigned) {
    std::fill(stamp_var.begin(), stamp_var.end(), 0);
    std::fill(stamp_tab.begin(), stamp_tab.end(), 0);
    std::fill(inq.begin(), inq.end(), 0);
    t = 0;
    qh = qt = 0;
    num_delete = 0;
    fail_c = -1;
    for (int v : evt) insert(v);
    while (qh != qt) {
      const int x = pop();
      for (int c : N.subs[x]) {
        if (stamp_var[x] > stamp_tab[c]) {
          for (int y : N.scope[c]) {
            if (assigned && assigned[y]) continue;
            bool aa = false;
            for (int z : N.scope[c])
              if (z != x && stamp_var[z] > stamp_tab[c]) aa = true;
            if (y != x || aa) {
              if (revise(D, c, y)) {
                if (dsize(D, N.W, y) == 0) {
                  fail_c = c;
                  return false;
                }
                insert(y);
              }
            }
          }
          ++t;
          stamp_tab[c] = t;
        }
      }
    }
    return true;
  }
};

// ---------------------------------------------------------------------------
// GAC for mixed arity. The reference's generic AC3 is wrong on networks that
// mix arities (AC::AC sizes its probe tuple to max_arity, src/AC.cpp:5, so
// Tabular::sat's binary_search, src/Network.cpp:310-312, never matches a
// binary table) and AC3bit refuses arity != 2 (src/AC3bit.cpp:4-6). This
// restates the GAC definition the reference's verifier uses
// (samples/verify_gac.cpp:121-164: a value stays iff every constraint on its
// variable has a tuple with that value whose other coordinates are all in the
// current domains) as a constraint worklist: binary constraints are revised in
// both directions with support rows, tables by projecting their valid tuples.
// ---------------------------------------------------------------------------
struct GAC {
  const Net& N;
  std::vector<int> q;
  std::vector<char> inq;
  size_t qh = 0, qt = 0;
  std::vector<u64> proj;
  int64_t num_delete = 0;
  explicit GAC(const Net& net) : N(net), q(net.nc + 1), inq(net.nc) {}
  void push(int c) {
    if (!inq[c]) {
      inq[c] = 1;
      q[qt] = c;
      qt = (qt + 1) % q.size();
    }
  }
  // Returns -1 on wipe-out, else 0; changed vars get their constraints queued.
  int apply(u64* D, int x, const u64* keep) {
    bool changed = false, empty = true;
    for (int w = 0; w < N.W; ++w) {
      u64& d = D[size_t(x) * N.W + w];
      const u64 nd = d & keep[w];
      if (nd != d) {
        num_delete += __builtin_popcountll(d & ~nd);
        d = nd;
        changed = true;
      }
      empty &= nd == 0;
    }
    if (empty) return -1;
    if (changed)
      for (int c : N.subs[x]) push(c);
    return 0;
  }
  int revise(u64* D, int c) {
    const int W = N.W;
    proj.assign(size_t(N.arity[c]) * W, 0);
    if (c < N.nb) {
      for (int pos = 0; pos < 2; ++pos) {
        const int v = N.scope[c][pos], o = N.scope[c][1 - pos];
        std::fill(proj.begin(), proj.begin() + W, 0);
        for (int a = 0; a < N.dom[v]; ++a) {
          if (!have(D, W, v, a)) continue;
          const u64* row = &N.bsup[pos][c][size_t(a) * W];
          for (int w = 0; w < W; ++w)
            if (row[w] & D[size_t(o) * W + w]) {
              proj[a >> 6] |= 1ull << (a & 63);
              break;
            }
        }
        if (apply(D, v, proj.data()) < 0) return -1;
      }
      return 0;
    }
    const int r = N.arity[c];
    const int* tp = N.tup[c];
    for (int k = 0; k < N.ntup[c]; ++k) {
      const int* tu = tp + size_t(k) * r;
      bool valid = true;
      for (int i = 0; i < r && valid; ++i) valid = have(D, W, N.scope[c][i], tu[i]);
      if (!valid) continue;
      for (int i = 0; i < r; ++i) proj[size_t(i) * W + (tu[i] >> 6)] |= 1ull << (tu[i] & 63);
    }
    for (int i = 0; i < r; ++i)
      if (apply(D, N.scope[c][i], &proj[size_t(i) * W]) < 0) return -1;
    return 0;
  }
  // evt empty => every constraint is queued.
  bool enforce(u64* D, const std::vector<int>& evt) {
    std::fill(inq.begin(), inq.end(), 0);
    qh = qt = 0;
    num_delete = 0;
    if (evt.empty()) {
      for (int c = 0; c < N.nc; ++c) push(c);
    } else {
      for (int x : evt)
        for (int c : N.subs[x]) push(c);
    }
    while (qh != qt) {
      const int c = q[qh];
      qh = (qh + 1) % q.size();
      inq[c] = 0;
      if (revise(D, c) < 0) return false;
    }
    return true;
  }
};

// One propagator: AC3bit on binary networks (the reference's AC_3bit), GAC
// when tables are present.
struct Prop {
  const Net& N;
  AC3bit ac;
  GAC gac;
  explicit Prop(const Net& net) : N(net), ac(net), gac(net) {}
  bool enforce(u64* D, const std::vector<int>& evt, const char* assigned, int64_t* dels) {
    bool ok;
    if (N.nt == 0) {
      ok = ac.enforce(D, evt, assigned);
      if (dels) *dels = ac.num_delete;
    } else {
      ok = gac.enforce(D, evt.size() == size_t(N.n) ? std::vector<int>() : evt);
      if (dels) *dels = gac.num_delete;
    }
    return ok;
  }
};

std::vector<int> all_vars(int n) {
  std::vector<int> v(n);
  for (int i = 0; i < n; ++i) v[i] = i;
  return v;
}

// ---------------------------------------------------------------------------
// SAC1: restates SAC1::enforce (src/SAC1.cpp:57-103), Gauss-Seidel order over
// variables and values, the singleton test on a scratch level.
// ---------------------------------------------------------------------------
bool sac1(const Net& N, u64* D, int64_t* deletions) {
  Prop P(N);
  int64_t del = 0, d = 0;
  std::vector<int> evt = all_vars(N.n);
  bool ok = P.enforce(D, evt, nullptr, &d);
  del += d;
  if (!ok) {
    *deletions = del;
    return false;
  }
  std::vector<u64> tmp(size_t(N.n) * N.W);
  std::vector<char> assigned(N.n, 0);
  bool modified;
  do {
    modified = false;
    for (int x = 0; x < N.n; ++x) {
      for (int a = 0; a < N.dom[x]; ++a) {
        if (!have(D, N.W, x, a)) continue;
        std::copy(D, D + tmp.size(), tmp.begin());
        reduce_to(tmp.data(), N.W, x, a);
        assigned[x] = 1;
        const bool res = P.enforce(tmp.data(), {x}, assigned.data(), nullptr);
        assigned[x] = 0;
        if (!res) {
          ++del;
          del_bit(D, N.W, x, a);
          ok = P.enforce(D, {x}, nullptr, &d);
          del += d;
          if (!ok) {
            *deletions = del;
            return false;
          }
          modified = true;
        }
      }
    }
  } while (modified);
  *deletions = del;
  return true;
}

// ---------------------------------------------------------------------------
// MAC with dom/min (or dom/deg) variable order and min value order: restates
// MAC::enforce (src/MAC.cpp:100-165), select_var VRH_DOM_MIN (:357-365) and
// VRH_DOM_DEG_MIN (:371-386), select_val
// VLH_MIN (:423-425), get_solution (:256-271), the level operations of
// Network / IntVar (src/Network.cpp:106-118, 235-256, 438-455) and
// AssignedStack push / pop / update_model_assigned (src/Solver.cpp:36-56,
// 114-116). The per-level "assigned" flags are kept exactly, because the
// variable order depends on them.
// ---------------------------------------------------------------------------
struct MacState {
  const Net& N;
  int L;
  std::vector<u64> dom;         // L levels of n*W words
  std::vector<char> assigned;   // L levels of n flags
  std::vector<int> top;         // per variable
  std::vector<std::pair<int, int>> I;
  MacState(const Net& net, const u64* d0) : N(net), L(net.n + 3) {
    dom.assign(size_t(L) * N.n * N.W, 0);
    std::copy(d0, d0 + size_t(N.n) * N.W, dom.begin());
    assigned.assign(size_t(L) * N.n, 0);
    top.assign(N.n, 0);
  }
  u64* D(int p) { return &dom[size_t(p) * N.n * N.W]; }
  char* A(int p) { return &assigned[size_t(p) * N.n]; }
  void new_level(int src) {
    std::copy(D(src), D(src) + size_t(N.n) * N.W, D(src + 1));
    std::copy(A(src), A(src) + N.n, A(src + 1));
    std::fill(top.begin(), top.end(), src);
  }
  void back_to(int dest) {
    for (int v = 0; v < N.n; ++v) {
      for (int i = dest; i <= top[v]; ++i) A(i)[v] = 0;
      top[v] = dest;
    }
  }
  void push(int v, int a) {
    I.emplace_back(v, a);
    A(int(I.size()))[v] = 1;
  }
  std::pair<int, int> pop() {
    auto va = I.back();
    I.pop_back();
    A(int(I.size()))[va.first] = 0;
    return va;
  }
  void update_model_assigned() {
    for (auto& va : I) A(int(I.size()))[va.first] = 1;
  }
};

// Number of distinct other variables sharing a constraint with each variable:
// the size of Network::neighborhood (get_neighbor, src/Network.cpp:467-476).
std::vector<int> neighbour_counts(const Net& N) {
  std::vector<int> cnt(N.n, 0);
  std::vector<int> mark(N.n, -1);
  for (int v = 0; v < N.n; ++v)
    for (int c : N.subs[v])
      for (int x : N.scope[c])
        if (x != v && mark[x] != v) {
          mark[x] = v;
          ++cnt[v];
        }
  return cnt;
}

// varh: 1 = VRH_DOM_MIN, 4 = VRH_DOM_DEG_MIN, 6 = VRH_DOM_WDEG_MIN
// (Heuristic::Var, include/Solver.h:55-63). dom/wdeg: every AC call that
// wipes a domain out adds 1 to the weight (initially 1, src/Network.cpp:303)
// of the constraint whose revision emptied it first in AC3::enforce's order
// (src/AC3.cpp:122-128); a variable's score is |D(x)| over the summed weights
// of its constraints with another unassigned variable, -1 when |D(x)| = 1 or
// the sum is 0 (src/MAC.cpp:387-408).
int mac(const Net& N, const u64* d0, int64_t time_limit_ms, int varh, int64_t* npos, int64_t* nneg, int* solution) {
  const auto t0 = std::chrono::steady_clock::now();
  auto elapsed_ms = [&]() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  };
  MacState S(N, d0);
  Prop P(N);
  const std::vector<int> deg = varh == 4 ? neighbour_counts(N) : std::vector<int>();
  std::vector<double> weight(varh == 6 ? N.nc : 0, 1.0);
  auto propagate = [&](u64* D, const std::vector<int>& evt, const char* A) {
    const bool ok = P.enforce(D, evt, A, nullptr);
    if (!ok && varh == 6 && P.ac.fail_c >= 0) weight[P.ac.fail_c] += 1.0;
    return ok;
  };
  *npos = *nneg = 0;
  if (!propagate(S.D(0), all_vars(N.n), S.A(0))) return 0;
  for (;;) {
    if (elapsed_ms() > double(time_limit_ms)) return 2;
    const int p = int(S.I.size());
    int var = -1;
    double min_size = 1e300;
    for (int v = 0; v < N.n; ++v) {
      if (S.A(p)[v]) continue;
      // dom/deg: integer size / |neighbourhood|, -1 for a variable without
      // neighbours; every order takes the first strict minimum.
      double key;
      if (varh == 6) {
        double w = 0.0;
        for (int c : N.subs[v]) {
          int free = 0;
          for (int y : N.scope[c]) free += S.A(p)[y] ? 0 : 1;
          if (free > 1) w += weight[c];
        }
        const int sz = dsize(S.D(p), N.W, v);
        key = (sz == 1 || w == 0.0) ? -1.0 : sz / w;
      } else {
        key = varh == 4 ? (deg[v] == 0 ? -1 : dsize(S.D(p), N.W, v) / deg[v]) : dsize(S.D(p), N.W, v);
      }
      if (key < min_size) {
        min_size = key;
        var = v;
      }
    }
    const int a = head(S.D(p), N.W, var);
    S.new_level(p);
    S.push(var, a);
    ++*npos;
    const int lv = int(S.I.size());
    reduce_to(S.D(lv), N.W, var, a);
    S.A(lv)[var] = 1;
    bool consistent = propagate(S.D(lv), {var}, S.A(lv));
    if (consistent && int(S.I.size()) == N.n) {
      for (int v = 0; v < N.n; ++v) solution[v] = head(S.D(lv), N.W, v);
      return 1;
    }
    while (!consistent && !S.I.empty()) {
      auto va = S.pop();
      const int q = int(S.I.size());
      S.back_to(q);
      del_bit(S.D(q), N.W, va.first, va.second);
      ++*nneg;
      consistent = dsize(S.D(q), N.W, va.first) > 0 && propagate(S.D(q), {va.first}, S.A(q));
      S.update_model_assigned();
    }
    if (!consistent) return 0;
  }
}

// ---------------------------------------------------------------------------
// d-way search of GModelSolver: restates GModelSolver::Solve / Search
// (src/GModelSolver.cu:31-189) with GModel::GetMinDomainVar
// (src/GModel.cu:1553-1572: the first variable of smallest domain size above
// one; -1 when every domain is a singleton). Every value of that variable in
// increasing order opens a child level: one positive node each, one negative
// node for each child whose GAC fixpoint wipes a domain out. The first
// solution stops the search. The propagator is the unique AC / GAC closure.
// ---------------------------------------------------------------------------
struct DWay {
  const Net& N;
  Prop P;
  std::chrono::steady_clock::time_point t0;
  int64_t limit_ms, npos = 0, nneg = 0;
  bool timed_out = false;
  std::vector<std::vector<u64>> levels;
  DWay(const Net& net, int64_t lim) : N(net), P(net), t0(std::chrono::steady_clock::now()), limit_ms(lim) {}

  int min_domain_var(const u64* D) const {
    int var = -1, best = 1 << 30;
    for (int v = 0; v < N.n; ++v) {
      const int sz = dsize(D, N.W, v);
      if (sz > 1 && sz < best) {
        best = sz;
        var = v;
      }
    }
    return var;
  }
  bool fully_assigned(const u64* D) const {
    for (int v = 0; v < N.n; ++v)
      if (dsize(D, N.W, v) != 1) return false;
    return true;
  }
  // Returns true to stop (solution found or time out); the solution is then
  // levels[level].
  bool search(int level, int* solution) {
    if (limit_ms > 0 &&
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count() >= limit_ms) {
      timed_out = true;
      return true;
    }
    const u64* D = levels[level].data();
    const int var = min_domain_var(D);
    if (var < 0) {
      if (!fully_assigned(D)) return false;
      for (int v = 0; v < N.n; ++v) solution[v] = head(D, N.W, v);
      return true;
    }
    if (int(levels.size()) <= level + 1) levels.emplace_back(size_t(N.n) * N.W);
    for (int a = 0; a < N.dom[var]; ++a) {
      if (!have(levels[level].data(), N.W, var, a)) continue;
      std::vector<u64>& child = levels[level + 1];
      std::copy(levels[level].begin(), levels[level].end(), child.begin());
      ++npos;
      reduce_to(child.data(), N.W, var, a);
      if (!P.enforce(child.data(), {var}, nullptr, nullptr)) {
        ++nneg;
        continue;
      }
      if (search(level + 1, solution)) return true;
    }
    return false;
  }
};

bool satisfied(const Net& N, int c, const int* val) {
  if (c < N.nb) {
    const int a = val[N.scope[c][0]], b = val[N.scope[c][1]];
    return (N.bsup[0][c][size_t(a) * N.W + (b >> 6)] >> (b & 63)) & 1ull;
  }
  const int r = N.arity[c];
  for (int k = 0; k < N.ntup[c]; ++k) {
    bool eq = true;
    for (int i = 0; i < r && eq; ++i) eq = N.tup[c][size_t(k) * r + i] == val[N.scope[c][i]];
    if (eq) return true;
  }
  return false;
}

bool singleton(const Net& N, Prop& P, const u64* D, std::vector<u64>& tmp, std::vector<char>& asg, int x, int a) {
  std::copy(D, D + size_t(N.n) * N.W, tmp.begin());
  reduce_to(tmp.data(), N.W, x, a);
  asg[x] = 1;
  const bool ok = P.enforce(tmp.data(), {x}, asg.data(), nullptr);
  asg[x] = 0;
  return ok;
}

}  // namespace

extern "C" {

int orc_ac3bit(const OrcNet* v, uint64_t* dom, int64_t* deletions) {
  if (v->nt != 0) return -1;
  Net N = build_net(v);
  AC3bit ac(N);
  const bool ok = ac.enforce(dom, all_vars(N.n), nullptr);
  if (deletions) *deletions = ac.num_delete;
  return ok ? 1 : 0;
}

int orc_gac(const OrcNet* v, uint64_t* dom, int64_t* deletions) {
  Net N = build_net(v);
  GAC g(N);
  const bool ok = g.enforce(dom, {});
  if (deletions) *deletions = g.num_delete;
  return ok ? 1 : 0;
}

// Literal restatement of CorrectGAC::ComputeGACDomains
// (samples/verify_gac.cpp:84-118) with IsGACConsistentWithDomains /
// HasSupportWithDomains (:121-164): tuple scans, variables in order, each
// variable's new domain installed before the next is checked, until no change.
// Binary relations are enumerated as their allowed tuple lists.
int orc_gac_definitional(const OrcNet* v, uint64_t* dom) {
  Net N = build_net(v);
  const int W = N.W;
  std::vector<std::vector<int>> bt(N.nb);
  for (int c = 0; c < N.nb; ++c)
    for (int a = 0; a < N.dom[N.scope[c][0]]; ++a)
      for (int b = 0; b < N.dom[N.scope[c][1]]; ++b)
        if ((N.bsup[0][c][size_t(a) * W + (b >> 6)] >> (b & 63)) & 1ull) {
          bt[c].push_back(a);
          bt[c].push_back(b);
        }
  auto has_support = [&](int c, int x, int a) {
    int pos = -1;
    for (int i = 0; i < N.arity[c]; ++i)
      if (N.scope[c][i] == x) {
        pos = i;
        break;
      }
    const int r = N.arity[c];
    const int* tp = c < N.nb ? bt[c].data() : N.tup[c];
    const int nt = c < N.nb ? int(bt[c].size() / 2) : N.ntup[c];
    for (int k = 0; k < nt; ++k) {
      const int* tu = tp + size_t(k) * r;
      if (tu[pos] != a) continue;
      bool valid = true;
      for (int i = 0; i < r && valid; ++i)
        if (i != pos) valid = have(dom, W, N.scope[c][i], tu[i]);
      if (valid) return true;
    }
    return false;
  };
  bool changed = true;
  while (changed) {
    changed = false;
    for (int x = 0; x < N.n; ++x) {
      for (int a = 0; a < N.dom[x]; ++a) {
        if (!have(dom, W, x, a)) continue;
        bool ok = true;
        for (int c : N.subs[x])
          if (!has_support(c, x, a)) {
            ok = false;
            break;
          }
        if (!ok) {
          del_bit(dom, W, x, a);
          changed = true;
        }
      }
    }
  }
  for (int x = 0; x < N.n; ++x)
    if (dsize(dom, W, x) == 0) return 0;
  return 1;
}

int orc_sac1(const OrcNet* v, uint64_t* dom, int64_t* deletions) {
  Net N = build_net(v);
  int64_t d = 0;
  const bool ok = sac1(N, dom, &d);
  if (deletions) *deletions = d;
  return ok ? 1 : 0;
}

int orc_mac(const OrcNet* v, const uint64_t* dom0, int64_t time_limit_ms, int64_t* num_positive,
            int64_t* num_negative, int* solution) {
  Net N = build_net(v);
  return mac(N, dom0, time_limit_ms, 1, num_positive, num_negative, solution);
}

int orc_mac_h(const OrcNet* v, const uint64_t* dom0, int64_t time_limit_ms, int varh, int64_t* num_positive,
              int64_t* num_negative, int* solution) {
  if (varh != 1 && varh != 4 && varh != 6) return -1;
  Net N = build_net(v);
  if (varh == 6 && N.nt) return -1;  // weights follow the binary AC3bit order only
  return mac(N, dom0, time_limit_ms, varh, num_positive, num_negative, solution);
}

int orc_dway(const OrcNet* v, const uint64_t* dom0, int64_t time_limit_ms, int64_t* num_positive,
             int64_t* num_negative, int* solution) {
  Net N = build_net(v);
  DWay S(N, time_limit_ms);
  S.levels.emplace_back(dom0, dom0 + size_t(N.n) * N.W);
  int status;
  if (!S.P.enforce(S.levels[0].data(), all_vars(N.n), nullptr, nullptr)) {
    status = 0;
  } else {
    const bool stop = S.search(0, solution);
    status = S.timed_out ? 2 : (stop ? 1 : 0);
  }
  *num_positive = S.npos;
  *num_negative = S.nneg;
  return status;
}

// Lexicographic backtracking that checks each constraint once its scope is
// fully assigned, in the spirit of the reference's BruteForceSolver
// (samples/verify_search.cpp:26-93), capped by the size of the search space.
int orc_brute_solve(const OrcNet* v, const uint64_t* dom0, double limit) {
  Net N = build_net(v);
  double space = 1;
  for (int x = 0; x < N.n; ++x) space *= std::max(1, dsize(dom0, N.W, x));
  if (space > limit) return -1;
  std::vector<std::vector<int>> closes(N.n);  // constraints whose last scope var is x
  for (int c = 0; c < N.nc; ++c) closes[*std::max_element(N.scope[c].begin(), N.scope[c].end())].push_back(c);
  std::vector<int> val(N.n, -1);
  std::vector<int> stack_a(N.n + 1, -1);
  int x = 0;
  while (x >= 0) {
    if (x == N.n) return 1;
    int a = val[x] + 1;
    bool placed = false;
    for (; a < N.dom[x]; ++a) {
      if (!have(dom0, N.W, x, a)) continue;
      val[x] = a;
      bool ok = true;
      for (int c : closes[x])
        if (!satisfied(N, c, val.data())) {
          ok = false;
          break;
        }
      if (ok) {
        placed = true;
        break;
      }
    }
    if (placed) {
      ++x;
      if (x < N.n) val[x] = -1;
    } else {
      val[x] = -1;
      --x;
    }
  }
  return 0;
}

int orc_check_solution(const OrcNet* v, const int* solution) {
  Net N = build_net(v);
  for (int x = 0; x < N.n; ++x)
    if (solution[x] < 0 || solution[x] >= N.dom[x]) return 0;
  for (int c = 0; c < N.nc; ++c)
    if (!satisfied(N, c, solution)) return 0;
  return 1;
}

int orc_singleton(const OrcNet* v, const uint64_t* dom, int x, int a) {
  Net N = build_net(v);
  Prop P(N);
  std::vector<u64> tmp(size_t(N.n) * N.W);
  std::vector<char> asg(N.n, 0);
  return singleton(N, P, dom, tmp, asg, x, a) ? 1 : 0;
}

double orc_time_singletons(const OrcNet* v, const uint64_t* dom, int64_t count, int threads, int64_t* failed,
                           int64_t* done) {
  Net N = build_net(v);
  std::vector<std::pair<int, int>> live;
  for (int x = 0; x < N.n; ++x)
    for (int a = 0; a < N.dom[x]; ++a)
      if (have(dom, N.W, x, a)) live.emplace_back(x, a);
  std::vector<std::pair<int, int>> pick;
  if (count >= int64_t(live.size())) {
    pick = live;
  } else {
    for (int64_t i = 0; i < count; ++i) pick.push_back(live[size_t(i * int64_t(live.size()) / count)]);
  }
  if (threads < 1) threads = 1;
  std::atomic<int64_t> nfail{0};
  std::atomic<size_t> next{0};
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    pool.emplace_back([&]() {
      Prop P(N);
      std::vector<u64> tmp(size_t(N.n) * N.W);
      std::vector<char> asg(N.n, 0);
      int64_t f = 0;
      for (;;) {
        const size_t i = next.fetch_add(1);
        if (i >= pick.size()) break;
        f += singleton(N, P, dom, tmp, asg, pick[i].first, pick[i].second) ? 0 : 1;
      }
      nfail += f;
    });
  }
  for (auto& th : pool) th.join();
  const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (failed) *failed = nfail.load();
  if (done) *done = int64_t(pick.size());
  return s;
}

int64_t orc_singleton_verdicts(const OrcNet* v, const uint64_t* dom, int threads, uint64_t* verdict) {
  Net N = build_net(v);
  std::vector<std::pair<int, int>> live;
  for (int x = 0; x < N.n; ++x)
    for (int a = 0; a < N.dom[x]; ++a)
      if (have(dom, N.W, x, a)) live.emplace_back(x, a);
  std::vector<char> res(live.size(), 0);
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < std::max(1, threads); ++t) {
    pool.emplace_back([&]() {
      Prop P(N);
      std::vector<u64> tmp(size_t(N.n) * N.W);
      std::vector<char> asg(N.n, 0);
      for (;;) {
        const size_t i = next.fetch_add(1);
        if (i >= live.size()) break;
        res[i] = singleton(N, P, dom, tmp, asg, live[i].first, live[i].second) ? 1 : 0;
      }
    });
  }
  for (auto& th : pool) th.join();
  std::fill(verdict, verdict + size_t(N.n) * N.W, 0ull);
  int64_t failed = 0;
  for (size_t i = 0; i < live.size(); ++i) {
    if (!res[i]) {
      ++failed;
      continue;
    }
    const int x = live[i].first, a = live[i].second;
    verdict[size_t(x) * N.W + (a >> 6)] |= 1ull << (a & 63);
  }
  return failed;
}

// SAC closure in Jacobi order: the loop of SAC1::enforce (src/SAC1.cpp:57-103)
// with every test of a sweep run against the sweep-start domains. Singleton
// failure is monotone in the domains, so the greatest SAC sub-domain it
// reaches is the one the sequential loop reaches.
int orc_sac_jacobi(const OrcNet* v, uint64_t* dom, int threads, int64_t* deletions, int* sweeps) {
  Net N = build_net(v);
  Prop P(N);
  int64_t del = 0, d = 0;
  int sw = 0;
  bool ok = P.enforce(dom, all_vars(N.n), nullptr, &d);
  del += d;
  std::vector<u64> verdict(size_t(N.n) * N.W);
  while (ok) {
    ++sw;
    const int64_t failed = orc_singleton_verdicts(v, dom, threads, verdict.data());
    if (failed == 0) break;
    std::vector<int> evt;
    for (int x = 0; x < N.n; ++x) {
      bool changed = false;
      for (int w = 0; w < N.W; ++w) {
        const size_t i = size_t(x) * N.W + w;
        if (dom[i] != verdict[i]) changed = true;
        dom[i] = verdict[i];
      }
      if (changed) evt.push_back(x);
    }
    del += failed;
    ok = P.enforce(dom, evt, nullptr, &d);
    del += d;
  }
  if (deletions) *deletions = del;
  if (sweeps) *sweeps = sw;
  return ok ? 1 : 0;
}

double orc_time_ac(const OrcNet* v, const uint64_t* dom, int reps, int64_t* deletions) {
  Net N = build_net(v);
  Prop P(N);
  std::vector<u64> D(size_t(N.n) * N.W);
  double best = 1e300;
  for (int r = 0; r < std::max(1, reps); ++r) {
    std::copy(dom, dom + D.size(), D.begin());
    const auto t0 = std::chrono::steady_clock::now();
    int64_t d = 0;
    P.enforce(D.data(), all_vars(N.n), nullptr, &d);
    best = std::min(best, std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    if (deletions) *deletions = d;
  }
  return best;
}

void* orc_gen_binary(int n, int d, int64_t e, double p_lo, double p_hi, double remove, uint64_t seed) {
  return new cpgen::Instance(cpgen::random_binary(n, d, e, p_lo, p_hi, remove, seed));
}
void* orc_gen_mixed(int n, int d, int64_t e, double p_lo, double p_hi, int k3, int ntup, double remove,
                    uint64_t seed) {
  return new cpgen::Instance(cpgen::random_mixed(n, d, e, p_lo, p_hi, k3, ntup, remove, seed));
}
void* orc_gen_uneven(uint64_t seed, int n_lo, int n_hi, int d_cap) {
  return new cpgen::Instance(cpgen::uneven_instance(seed, n_lo, n_hi, d_cap));
}
void orc_gen_free(void* inst) { delete static_cast<cpgen::Instance*>(inst); }
const uint64_t* orc_gen_view(void* inst, OrcNet* out, uint64_t* fingerprint, int64_t* brows_words,
                             int64_t* ttup_ints, int64_t* tscope_ints) {
  auto* I = static_cast<cpgen::Instance*>(inst);
  out->n = I->n;
  out->W = I->W;
  out->dom = I->dom.data();
  out->nb = I->n_bin();
  out->bx = I->bx.data();
  out->by = I->by.data();
  out->brows = I->brows.data();
  out->nt = I->n_tab();
  out->tarity = I->tarity.data();
  out->tscope = I->tscope.data();
  out->tntup = I->tntup.data();
  out->ttup = I->ttup.data();
  if (fingerprint) *fingerprint = cpgen::fingerprint(*I);
  if (brows_words) *brows_words = int64_t(I->brows.size());
  if (ttup_ints) *ttup_ints = int64_t(I->ttup.size());
  if (tscope_ints) *tscope_ints = int64_t(I->tscope.size());
  return I->init.data();
}

}  // extern "C"
