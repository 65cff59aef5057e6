// GpuAC: the reference-side adapter that makes the GPU engine an `AC` of
// leezear2022/cpim (the abstract class of include/Solver.h:309-331), so that
// code written against AC::enforce(vector<IntVar*>& x_evt, int level) -- the
// SAC1 loop (src/SAC1.cpp:57-103), the MAC node loop (src/MAC.cpp:100-165) --
// runs its propagation on the device unchanged. A maintainer adds this header
// to the reference next to include/Solver.h and selects GpuAC where the MAC
// and SAC1 factories (src/MAC.cpp:14-40, src/SAC1.cpp:5-22) create AC3bit.
//
// It needs the reference's headers (Solver.h, Network.h) and this
// repository's include/cpgpu.h, and links libcpgpu.so; it has no CUDA code.
// Constraints of any arity: binary ones become support rows (AC3bit's,
// src/AC3bit.cpp:3-27), wider ones positive tables revised like the generic
// AC3 (src/AC3.cpp:195-209).
//
// Level protocol: the reference keeps n + 3 domain levels per IntVar
// (src/Network.cpp:78); the device network is uploaded with the same number
// of levels. enforce() pushes the host's level to the device, runs the AC
// fixpoint there (cp_enforce_ac, seeded with x_evt) and writes the closure
// back into IntVar::bitDom(level), so the host levels stay authoritative and
// the reference's CopyLevel / ReduceTo / BackTo work as before.
#ifndef CPIM_GB300_GPU_AC_HPP
#define CPIM_GB300_GPU_AC_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "Solver.h"
#include "cpgpu.h"

namespace cpim {

class GpuAC : public AC {
 public:
  explicit GpuAC(Network* m, int device = 0) : AC(m), n_(static_cast<int>(m->vars.size())), W_(m->max_bitDom_size()) {
    check(cp_engine_create(device, &e_), "cp_engine_create");
    std::vector<int> dom(n_);
    std::vector<uint64_t> init(static_cast<size_t>(n_) * W_);
    for (int x = 0; x < n_; ++x) {
      dom[x] = m->vars[x]->capacity();
      pack_var(x, 0, init.data());
    }
    // Support rows of each binary constraint's first variable over its
    // second: row a, bit b set iff (a, b) is an allowed tuple (the bitSup_
    // rows of src/AC3bit.cpp:11-26 for scope[0]; the device derives the other
    // side). Wider constraints keep their tuple lists.
    std::vector<int> scope, t_arity, t_scope, t_ntup, t_tuples;
    std::vector<uint64_t> rows;
    for (Tabular* c : m->tabs) {
      if (c->scope.size() != 2) {
        t_arity.push_back(static_cast<int>(c->scope.size()));
        for (IntVar* v : c->scope) t_scope.push_back(v->id());
        t_ntup.push_back(static_cast<int>(c->tuples().size()));
        for (const auto& t : c->tuples()) t_tuples.insert(t_tuples.end(), t.begin(), t.end());
        continue;
      }
      IntVar* x = c->scope[0];
      IntVar* y = c->scope[1];
      scope.push_back(x->id());
      scope.push_back(y->id());
      const size_t base = rows.size();
      rows.resize(base + static_cast<size_t>(x->capacity()) * W_, 0ull);
      for (const auto& t : c->tuples()) rows[base + static_cast<size_t>(t[0]) * W_ + (t[1] >> 6)] |= 1ull << (t[1] & 63);
    }
    check(cp_net_upload(e_, n_, dom.data(), W_, init.data(), static_cast<int>(scope.size() / 2), scope.data(),
                        rows.data(), static_cast<int>(t_arity.size()), t_arity.data(), t_scope.data(), t_ntup.data(),
                        t_tuples.data(), n_ + 3, &net_),
          "cp_net_upload");
    buf_.resize(static_cast<size_t>(n_) * W_);
  }
  ~GpuAC() override {
    if (net_) cp_net_destroy(net_);
    if (e_) cp_engine_destroy(e_);
  }
  GpuAC(const GpuAC&) = delete;
  GpuAC& operator=(const GpuAC&) = delete;

  ConsistencyState enforce(vector<IntVar*>& x_evt, int level) override {
    for (int x = 0; x < n_; ++x) pack_var(x, level, buf_.data());
    check(cp_dom_set(net_, level, buf_.data()), "cp_dom_set");
    std::vector<int> evt;
    evt.reserve(x_evt.size());
    for (IntVar* v : x_evt) evt.push_back(v->id());
    cp_stats st{};
    check(cp_enforce_ac(net_, level, static_cast<int>(evt.size()), evt.empty() ? nullptr : evt.data(), &st),
          "cp_enforce_ac");
    ConsistencyState res;
    res.state = st.inconsistent == 0;
    res.num_delete = static_cast<int>(st.deletions);
    res.level = level;
    if (res.state) {
      check(cp_dom_get(net_, level, buf_.data()), "cp_dom_get");
      for (int x = 0; x < n_; ++x) unpack_var(x, level, buf_.data());
    }
    delete_ += res.num_delete;
    cs = res;
    return res;
  }

 private:
  static void check(int rc, const char* what) {
    if (rc != 0) throw std::runtime_error(std::string(what) + ": " + cp_last_error_string());
  }
  void pack_var(int x, int level, uint64_t* out) {
    auto& bd = m_->vars[x]->bitDom(level);
    for (int w = 0; w < W_; ++w) out[static_cast<size_t>(x) * W_ + w] = w < static_cast<int>(bd.size()) ? bd[w].to_ullong() : 0ull;
  }
  void unpack_var(int x, int level, const uint64_t* in) {
    auto& bd = m_->vars[x]->bitDom(level);
    for (int w = 0; w < static_cast<int>(bd.size()) && w < W_; ++w) bd[w] = in[static_cast<size_t>(x) * W_ + w];
  }

  int n_, W_;
  cp_engine* e_ = nullptr;
  cp_net* net_ = nullptr;
  std::vector<uint64_t> buf_;
};

}  // namespace cpim

#endif  // CPIM_GB300_GPU_AC_HPP
