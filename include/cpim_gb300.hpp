// C++ facade of the reference's host API over the cpgpu C ABI (cpgpu.h), so
// host code written against leezear2022/cpim's Network / AC / SAC1 / MAC /
// GModel / GModelSolver classes can run its propagation on a GB300.
//
// Names, enums and method signatures follow the reference:
//   ACAlgorithm, Heuristic::Var/Val        include/Solver.h:13-69
//   SearchStatistics, ConsistencyState      include/Solver.h:71-97
//   AC::enforce(x_evt, level)               include/Solver.h:309-331
//   SAC1(n, a).enforce(x_evt, level), del() include/Solver.h:422-437
//   MAC(n, ac, varh, valh).enforce(ms)      include/Solver.h:575-606
//   GacStats, GModel level/search API       include/GModel.cuh:17-21, 184-253
//   GpuSearchStatistics, GModelSolver       include/GModelSolver.h:11-70
// The model is described with ModelBuilder (a small stand-in for the
// reference's model::ModelBuilder, include/model/model_builder.h:101-172):
// variables with domain sizes, extension constraints with support or conflict
// tuples. Binary constraints become support bit-rows, higher-arity tables stay
// tuple lists. Every propagation runs in the engine; there is no CPU path.
//
// Header-only; link with cpim_gb300/_build/libcpgpu.so.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "cpgpu.h"

namespace cpim_gb300 {

enum ACAlgorithm {
  CA_AC1, CA_AC2, AC_3, AC_4, AC_6, AC_7, AC_2001, AC_3bit, AC_3rm, STR_1, STR_2, STR_3,
  A_FC, A_FC_bit, A_NSAC, CA_LMRPC_BIT, CA_RPC3
};

namespace Heuristic {
enum Var { VRH_LEX, VRH_DOM_MIN, VRH_VWDEG, VRH_DEG_MIN, VRH_DOM_DEG_MIN, VRH_DOM_DDEG_MIN, VRH_DOM_WDEG_MIN };
enum Val { VLH_MIN, VLH_MIN_DOM, VLH_MIN_INC, VLH_MAX_INC, VLH_VWDEG };
}  // namespace Heuristic

struct SearchStatistics {
  uint64_t num_sol = 0;
  uint64_t num_positive = 0;
  uint64_t num_negative = 0;
  uint64_t nodes = 0;
  uint64_t build_time = 0;
  uint64_t solve_time = 0;
  uint64_t total_time = 0;
  bool time_out = false;
  bool pass = false;
};

struct ConsistencyState {
  bool state = true;
  int num_delete = 0;
  int var = -1;   // failing variable id when known
  int level = 0;
};

struct GacStats {
  int iterations = 0;
  int deletions = 0;
  bool inconsistent = false;
};

struct GpuSearchStatistics {
  int num_positive = 0;
  int num_negative = 0;
  int num_solutions = 0;
  int gac_iterations = 0;
  int gac_deletions = 0;
  bool time_out = false;
  bool unsolvable = false;
  double solve_time = 0.0;
  double gac_time = 0.0;
};

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc != CP_OK) throw Error(rc, std::string("cpgpu: ") + cp_last_error_string());
}

// One CUDA device and stream.
class Engine {
 public:
  explicit Engine(int device = 0) { check(cp_engine_create(device, &e_)); }
  ~Engine() { cp_engine_destroy(e_); }
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;
  cp_engine* get() const { return e_; }
  int64_t launches() const { return cp_engine_launches(e_); }

 private:
  cp_engine* e_ = nullptr;
};

// Model description (variables 0..n-1 with value indices 0..size-1).
class ModelBuilder {
 public:
  enum class Semantics { kSupports, kConflicts };
  int AddVariable(int domain_size) {
    if (domain_size < 1) throw Error(CP_E_ARG, "domain size must be positive");
    dom_.push_back(domain_size);
    return static_cast<int>(dom_.size()) - 1;
  }
  // Extension constraint (ExtensionConstraint, include/model/types.h:148-161).
  void AddExtension(Semantics sem, std::vector<int> scope, std::vector<std::vector<int>> tuples) {
    cons_.push_back({sem, std::move(scope), std::move(tuples)});
  }
  int num_variables() const { return static_cast<int>(dom_.size()); }

 private:
  friend class Network;
  struct Con {
    Semantics sem;
    std::vector<int> scope;
    std::vector<std::vector<int>> tuples;
  };
  std::vector<int> dom_;
  std::vector<Con> cons_;
};

// The network: device-resident domains (a level stack) and relations
// (Network, include/Network.h:324-380).
// A variable of the network, with the reference's id() (IntVar,
// include/Network.h:142-193). Domains stay on the device; read them through
// Network::Domains / Sizes.
class IntVar {
 public:
  explicit IntVar(int id) : id_(id) {}
  int id() const { return id_; }

 private:
  int id_;
};

class Network {
 public:
  // Network::vars (include/Network.h:127): the variables in id order, so that
  // reference code such as ac->enforce(net.vars, level) compiles unchanged.
  std::vector<IntVar*> vars;

  Network(Engine& engine, const ModelBuilder& model, int max_levels = 0) : n_(model.num_variables()) {
    var_store_.reserve(n_);
    for (int x = 0; x < n_; ++x) {
      var_store_.emplace_back(x);
      vars.push_back(&var_store_.back());
    }
    int maxd = 1;
    for (int d : model.dom_) maxd = d > maxd ? d : maxd;
    W_ = (maxd + 63) / 64;
    dom_ = model.dom_;
    std::vector<uint64_t> init(static_cast<size_t>(n_) * W_, 0);
    for (int x = 0; x < n_; ++x)
      for (int a = 0; a < dom_[x]; ++a) init[static_cast<size_t>(x) * W_ + (a >> 6)] |= 1ull << (a & 63);
    std::vector<int> bscope, tar, tsc, tnt, ttu;
    std::vector<uint64_t> rows;
    for (const auto& c : model.cons_) {
      for (int v : c.scope)
        if (v < 0 || v >= n_) throw Error(CP_E_ARG, "constraint scope out of range");
      const int r = static_cast<int>(c.scope.size());
      if (r == 2) {
        const int x = c.scope[0], y = c.scope[1];
        std::vector<uint64_t> block(static_cast<size_t>(dom_[x]) * W_, 0);
        if (c.sem == ModelBuilder::Semantics::kConflicts) {
          for (int a = 0; a < dom_[x]; ++a)
            for (int b = 0; b < dom_[y]; ++b) block[static_cast<size_t>(a) * W_ + (b >> 6)] |= 1ull << (b & 63);
        }
        for (const auto& t : c.tuples) {
          if (t.size() != 2 || t[0] < 0 || t[0] >= dom_[x] || t[1] < 0 || t[1] >= dom_[y]) continue;
          uint64_t& w = block[static_cast<size_t>(t[0]) * W_ + (t[1] >> 6)];
          if (c.sem == ModelBuilder::Semantics::kSupports)
            w |= 1ull << (t[1] & 63);
          else
            w &= ~(1ull << (t[1] & 63));
        }
        bscope.push_back(x);
        bscope.push_back(y);
        rows.insert(rows.end(), block.begin(), block.end());
      } else {
        if (c.sem != ModelBuilder::Semantics::kSupports)
          throw Error(CP_E_UNSUPPORTED, "non-binary conflict tables are not supported");
        tar.push_back(r);
        tsc.insert(tsc.end(), c.scope.begin(), c.scope.end());
        tnt.push_back(static_cast<int>(c.tuples.size()));
        for (const auto& t : c.tuples) {
          if (static_cast<int>(t.size()) != r) throw Error(CP_E_ARG, "tuple arity mismatch");
          ttu.insert(ttu.end(), t.begin(), t.end());
        }
      }
    }
    check(cp_net_upload(engine.get(), n_, dom_.data(), W_, init.data(), static_cast<int>(bscope.size() / 2),
                        bscope.data(), rows.data(), static_cast<int>(tar.size()), tar.data(), tsc.data(),
                        tnt.data(), ttu.data(), max_levels, &net_));
  }
  ~Network() { cp_net_destroy(net_); }
  Network(const Network&) = delete;
  Network& operator=(const Network&) = delete;

  cp_net* get() const { return net_; }
  int num_vars() const { return n_; }
  int words() const { return W_; }
  int capacity(int x) const { return dom_[x]; }
  // Level stack (Network::CopyLevel / NewLevel, src/Network.cpp:438-451).
  void CopyLevel(int src, int dest) { check(cp_level_copy(net_, src, dest)); }
  int NewLevel(int src) {
    CopyLevel(src, src + 1);
    return src + 1;
  }
  std::vector<uint64_t> Domains(int level) const {
    std::vector<uint64_t> out(static_cast<size_t>(n_) * W_);
    check(cp_dom_get(net_, level, out.data()));
    return out;
  }
  std::vector<int> Sizes(int level) const {
    std::vector<int> out(n_);
    check(cp_dom_sizes(net_, level, out.data()));
    return out;
  }
  void ReduceTo(int var, int a, int level) { check(cp_reduce_to(net_, level, var, a)); }
  void RemoveValue(int var, int a, int level) { check(cp_remove(net_, level, var, a)); }

 private:
  cp_net* net_ = nullptr;
  int n_ = 0, W_ = 1;
  std::vector<int> dom_;
  std::vector<IntVar> var_store_;
};

inline std::vector<int> var_ids(const std::vector<IntVar*>& vs) {
  std::vector<int> ids;
  ids.reserve(vs.size());
  for (const IntVar* v : vs) ids.push_back(v->id());
  return ids;
}

// AC::enforce(x_evt, level) (include/Solver.h:315): AC_3bit on binary
// networks, GAC with tables.
class AC {
 public:
  explicit AC(Network* n) : n_(n) {}
  virtual ~AC() = default;
  virtual ConsistencyState enforce(const std::vector<int>& x_evt, int level) {
    cp_stats st{};
    check(cp_enforce_ac(n_->get(), level, static_cast<int>(x_evt.size()), x_evt.empty() ? nullptr : x_evt.data(),
                        &st));
    cs.state = st.inconsistent == 0;
    cs.num_delete = static_cast<int>(st.deletions);
    cs.level = level;
    delete_ += cs.num_delete;
    last_ = st;
    return cs;
  }
  // The reference's signature (include/Solver.h:315).
  virtual ConsistencyState enforce(std::vector<IntVar*>& x_evt, int level) { return enforce(var_ids(x_evt), level); }
  int del() const { return delete_; }
  const cp_stats& last_stats() const { return last_; }
  ConsistencyState cs;

 protected:
  Network* n_;
  int delete_ = 0;
  cp_stats last_{};
};

class AC3bit : public AC {
 public:
  using AC::AC;
};

// SAC1 (include/Solver.h:422-437, src/SAC1.cpp:57-103).
class SAC1 {
 public:
  SAC1(Network* n, ACAlgorithm a) : n_(n) {
    if (a != AC_3bit && a != AC_3) throw Error(CP_E_UNSUPPORTED, "SAC1 runs over AC_3bit / AC_3");
  }
  bool enforce(const std::vector<int>& /*x_evt*/, int level) {
    cp_stats st{};
    check(cp_enforce_sac1(n_->get(), level, &st));
    del_ += static_cast<int>(st.deletions);
    last_ = st;
    return st.inconsistent == 0;
  }
  // The reference's signature (SAC1::enforce, include/Solver.h:425).
  bool enforce(std::vector<IntVar*> x_evt, int level) { return enforce(var_ids(x_evt), level); }
  int del() const { return del_; }
  const cp_stats& last_stats() const { return last_; }

 private:
  Network* n_;
  int del_ = 0;
  cp_stats last_{};
};

// MAC (include/Solver.h:575-606, src/MAC.cpp:100-165).
class MAC {
 public:
  MAC(Network* n, ACAlgorithm ac_algzm, Heuristic::Var varh, Heuristic::Val valh)
      : n_(n), varh_(varh), valh_(valh) {
    if (ac_algzm != AC_3bit && ac_algzm != AC_3) throw Error(CP_E_UNSUPPORTED, "MAC runs over AC_3bit / AC_3");
  }
  SearchStatistics enforce(int time_limits) {
    cp_search_result r{};
    std::vector<int> sol(n_->num_vars(), -1);
    check(cp_mac_solve(n_->get(), static_cast<int>(varh_), static_cast<int>(valh_), time_limits, &r, sol.data()));
    SearchStatistics s;
    s.num_positive = static_cast<uint64_t>(r.num_positive);
    s.num_negative = static_cast<uint64_t>(r.num_negative);
    s.num_sol = r.status == 1 ? 1 : 0;
    s.time_out = r.status == 2;
    s.solve_time = static_cast<uint64_t>(r.solve_ms);
    if (r.status == 1) {
      solution = sol;
      sol_str.clear();
      for (size_t i = 0; i < sol.size(); ++i) sol_str += (i ? " " : "") + std::to_string(sol[i]);
    }
    return s;
  }
  std::vector<int> solution;
  std::string sol_str;

 private:
  Network* n_;
  Heuristic::Var varh_;
  Heuristic::Val valh_;
};

// GModel: the reference GPU model's level and search-helper API
// (include/GModel.cuh:184-253) on the engine's level stack.
class GModel {
 public:
  explicit GModel(Network* n) : num_vars(n->num_vars()), n_(n) { refresh(0); }
  GacStats EnforceGAC(bool /*verbose*/ = true, int assigned_var = -1) {
    cp_stats st{};
    if (assigned_var >= 0)
      check(cp_enforce_ac(n_->get(), level_, 1, &assigned_var, &st));
    else
      check(cp_enforce_ac(n_->get(), level_, 0, nullptr, &st));
    refresh(level_);
    GacStats g;
    g.iterations = st.rounds;
    g.deletions = static_cast<int>(st.deletions);
    g.inconsistent = st.inconsistent != 0;
    return g;
  }
  GacStats EnforceGAC_Persistent(bool verbose = true, int assigned_var = -1) {
    return EnforceGAC(verbose, assigned_var);
  }
  int CreateNewLevel() {
    n_->CopyLevel(level_, level_ + 1);
    ++level_;
    refresh(level_);
    return level_;
  }
  void BackToLevel(int level) {
    if (level < 0 || level > level_) throw Error(CP_E_ARG, "BackToLevel: invalid level");
    level_ = level;
    refresh(level_);
  }
  int GetCurrentLevel() const { return level_; }
  bool AssignValue(int var, int value, int level) {
    n_->ReduceTo(var, value, level);
    if (level == level_) refresh(level_);
    return true;
  }
  bool RemoveValue(int var, int value, int level) {
    n_->RemoveValue(var, value, level);
    if (level == level_) refresh(level_);
    return sizes_at(level)[var] > 0;
  }
  int GetDomainSize(int var, int level) const { return sizes_at(level)[var]; }
  int GetMinDomainVar(int level) const {
    const std::vector<int> s = sizes_at(level);
    int best = -1, min_size = 1 << 30;
    for (int v = 0; v < num_vars; ++v)
      if (s[v] > 1 && s[v] < min_size) {
        min_size = s[v];
        best = v;
      }
    return best;
  }
  bool IsAssigned(int var, int level) const { return sizes_at(level)[var] == 1; }
  bool IsFullyAssigned(int level) const {
    for (int s : sizes_at(level))
      if (s != 1) return false;
    return true;
  }
  int GetAssignedValue(int var, int level) const { return IsAssigned(var, level) ? GetFirstValue(var, level) : -1; }
  int GetFirstValue(int var, int level) const { return GetNextValue(var, -1, level); }
  int GetNextValue(int var, int value, int level) const {
    const std::vector<uint64_t> d = level == level_ ? dom_ : n_->Domains(level);
    const int W = n_->words();
    for (int b = value + 1; b < n_->capacity(var); ++b)
      if ((d[static_cast<size_t>(var) * W + (b >> 6)] >> (b & 63)) & 1ull) return b;
    return -1;
  }
  Network* network() const { return n_; }
  const int num_vars;

 private:
  void refresh(int level) {
    dom_ = n_->Domains(level);
    sizes_ = n_->Sizes(level);
  }
  std::vector<int> sizes_at(int level) const { return level == level_ ? sizes_ : n_->Sizes(level); }
  Network* n_;
  int level_ = 0;
  std::vector<uint64_t> dom_;
  std::vector<int> sizes_;
};

// GModelSolver (include/GModelSolver.h:32-70): d-way search on the device.
class GModelSolver {
 public:
  explicit GModelSolver(GModel* model, bool verbose = false) : model_(model) {
    (void)verbose;
    if (!model_) throw Error(CP_E_ARG, "[GModelSolver] model is null!");
  }
  GpuSearchStatistics Solve(int time_limit = 0) {
    cp_search_result r{};
    std::vector<int> sol(model_->num_vars, -1);
    check(cp_gsolver_solve(model_->network()->get(), time_limit > 0 ? time_limit : (int64_t(1) << 40), &r,
                           sol.data()));
    GpuSearchStatistics s;
    s.num_positive = static_cast<int>(r.num_positive);
    s.num_negative = static_cast<int>(r.num_negative);
    s.num_solutions = r.status == 1 ? 1 : 0;
    s.time_out = r.status == 2;
    s.unsolvable = r.status == 0;
    s.solve_time = r.solve_ms / 1000.0;
    solutions_.clear();
    if (r.status == 1) solutions_.push_back(sol);
    return s;
  }
  std::vector<int> GetSolution() const { return solutions_.empty() ? std::vector<int>() : solutions_[0]; }
  std::vector<std::vector<int>> GetAllSolutions() const { return solutions_; }

 private:
  GModel* model_;
  std::vector<std::vector<int>> solutions_;
};

}  // namespace cpim_gb300
