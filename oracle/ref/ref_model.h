// The reference's model of a seeded instance (cpim_gb300/csrc/cp_gen.h): one
// domain per distinct size, every binary constraint and table as a positive
// extension constraint, built through the reference's ModelBuilder, and the
// instance's initial removals applied at level 0. Test infrastructure shared by
// the reference driver (oracle/ref/ref_driver.cpp) and the reference-side
// binding check (tests/cpp/gpu_ac_check.cpp).
#ifndef CPIM_ORACLE_REF_MODEL_H
#define CPIM_ORACLE_REF_MODEL_H

#include <cstdlib>
#include <iostream>
#include <string>
#include <vector>

#include "Network.h"
#include "cp_gen.h"
#include "model/model_builder.h"

namespace refmodel {

using namespace cpim;

inline model::IntermediateModel build_model(const cpgen::Instance& I) {
  model::ModelBuilder b("generated");
  std::vector<model::DomainId> dom_ids;
  std::vector<int> dom_size_of_id;
  std::vector<model::VariableId> vars;
  for (int x = 0; x < I.n; ++x) {
    int found = -1;
    for (size_t k = 0; k < dom_size_of_id.size(); ++k)
      if (dom_size_of_id[k] == I.dom[x]) found = int(k);
    if (found < 0) {
      dom_ids.push_back(b.AddDomain("D" + std::to_string(I.dom[x])).WithRange(0, I.dom[x] - 1).Build());
      dom_size_of_id.push_back(I.dom[x]);
      found = int(dom_ids.size()) - 1;
    }
    vars.push_back(b.AddVariable("x" + std::to_string(x)).WithDomain(dom_ids[found]).Build());
  }
  for (int c = 0; c < I.n_bin(); ++c) {
    std::vector<std::vector<int>> tuples;
    const int x = I.bx[c], y = I.by[c];
    for (int a = 0; a < I.dom[x]; ++a) {
      const uint64_t* r = I.row(c, a);
      for (int bv = 0; bv < I.dom[y]; ++bv)
        if ((r[bv >> 6] >> (bv & 63)) & 1ull) tuples.push_back({a, bv});
    }
    b.AddConstraint().AsExtension(model::ExtensionConstraint::Semantics::kSupports,
                                  {vars[x], vars[y]}, std::move(tuples)).Build();
  }
  for (int t = 0; t < I.n_tab(); ++t) {
    const int r = I.tarity[t];
    std::vector<model::VariableId> scope;
    for (int i = 0; i < r; ++i) scope.push_back(vars[I.tscope[I.tscope_off[t] + i]]);
    std::vector<std::vector<int>> tuples(I.tntup[t], std::vector<int>(r));
    for (int k = 0; k < I.tntup[t]; ++k)
      for (int i = 0; i < r; ++i) tuples[k][i] = I.ttup[I.ttup_off[t] + int64_t(k) * r + i];
    b.AddConstraint().AsExtension(model::ExtensionConstraint::Semantics::kSupports, scope,
                                  std::move(tuples)).Build();
  }
  auto m = std::move(b).Build();
  if (!m.ok()) {
    std::cerr << "model build failed: " << m.status().message() << std::endl;
    std::exit(2);
  }
  return std::move(m).value();
}

inline void apply_initial_domains(Network& net, const cpgen::Instance& I) {
  for (int x = 0; x < I.n; ++x)
    for (int a = 0; a < I.dom[x]; ++a)
      if (!I.bit(x, a)) net.vars[x]->RemoveValue(a, 0);
}

}  // namespace refmodel

#endif
