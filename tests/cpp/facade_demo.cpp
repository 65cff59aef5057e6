// Drives the C++ facade (include/cpim_gb300.hpp) the way the reference's host
// code drives cpim: build a model, construct a Network, run AC3bit, SAC1, MAC
// with dom/min + min value, and GModel + GModelSolver; print one JSON object
// per run. Built and run by tests/test_gpu_facade.py.
//
// Usage: facade_demo N D E P REMOVE SEED
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "cpim_gb300.hpp"

using namespace cpim_gb300;

// Initial domains of the generated instance; removals are applied through the
// level API (IntVar::RemoveValue at level 0), as the reference's drivers do.
static std::vector<uint64_t> g_init;
static int g_W = 1;

static ModelBuilder model_from_generator(int n, int d, long e, double p, double remove, unsigned long long seed) {
  cp_instance* inst = nullptr;
  check(cp_gen_binary(n, d, e, p, p, remove, seed, &inst));
  int64_t sz[8];
  check(cp_gen_sizes(inst, sz));
  const int W = static_cast<int>(sz[1]), nb = static_cast<int>(sz[2]);
  std::vector<int> dom(n), scope(2 * nb);
  std::vector<uint64_t> init(static_cast<size_t>(n) * W), rows(static_cast<size_t>(sz[4]));
  check(cp_gen_export(inst, dom.data(), init.data(), scope.data(), rows.data(), nullptr, nullptr, nullptr, nullptr));
  cp_gen_free(inst);
  ModelBuilder b;
  for (int x = 0; x < n; ++x) b.AddVariable(dom[x]);
  size_t off = 0;
  for (int c = 0; c < nb; ++c) {
    const int x = scope[2 * c], y = scope[2 * c + 1];
    std::vector<std::vector<int>> tuples;
    for (int a = 0; a < dom[x]; ++a)
      for (int v = 0; v < dom[y]; ++v)
        if ((rows[off + static_cast<size_t>(a) * W + (v >> 6)] >> (v & 63)) & 1ull) tuples.push_back({a, v});
    off += static_cast<size_t>(dom[x]) * W;
    b.AddExtension(ModelBuilder::Semantics::kSupports, {x, y}, tuples);
  }
  g_init = init;
  g_W = W;
  return b;
}

static void apply_init(Network& net) {
  for (int x = 0; x < net.num_vars(); ++x)
    for (int a = 0; a < net.capacity(x); ++a)
      if (!((g_init[static_cast<size_t>(x) * g_W + (a >> 6)] >> (a & 63)) & 1ull)) net.RemoveValue(x, a, 0);
}

static std::string hex(const std::vector<uint64_t>& d) {
  std::string s;
  char buf[17];
  for (uint64_t w : d) {
    std::snprintf(buf, sizeof buf, "%016llx", static_cast<unsigned long long>(w));
    s += buf;
  }
  return s;
}

int main(int argc, char** argv) {
  if (argc < 7) return 2;
  const int n = std::atoi(argv[1]), d = std::atoi(argv[2]);
  const long e = std::atol(argv[3]);
  const double p = std::atof(argv[4]), rm = std::atof(argv[5]);
  const unsigned long long seed = std::strtoull(argv[6], nullptr, 10);
  Engine engine(0);
  ModelBuilder model = model_from_generator(n, d, e, p, rm, seed);
  {
    Network net(engine, model);
    apply_init(net);
    AC3bit ac(&net);
    ConsistencyState cs = ac.enforce(net.vars, 0);  // AC::enforce(vector<IntVar*>&, int)
    std::printf("{\"op\": \"ac3bit\", \"consistent\": %s, \"deletions\": %d, \"domains\": \"%s\"}\n",
                cs.state ? "true" : "false", cs.num_delete, hex(net.Domains(0)).c_str());
  }
  {
    Network net(engine, model);
    apply_init(net);
    SAC1 sac(&net, AC_3bit);
    const bool ok = sac.enforce(net.vars, 0);  // SAC1::enforce(vector<IntVar*>, int)
    std::printf("{\"op\": \"sac1\", \"consistent\": %s, \"deletions\": %d, \"domains\": \"%s\"}\n",
                ok ? "true" : "false", sac.del(), hex(net.Domains(0)).c_str());
  }
  {
    Network net(engine, model);
    apply_init(net);
    MAC mac(&net, AC_3bit, Heuristic::VRH_DOM_MIN, Heuristic::VLH_MIN);
    SearchStatistics st = mac.enforce(60000);
    std::printf("{\"op\": \"mac\", \"num_positive\": %llu, \"num_negative\": %llu, \"num_sol\": %llu, \"solution\": [%s]}\n",
                static_cast<unsigned long long>(st.num_positive), static_cast<unsigned long long>(st.num_negative),
                static_cast<unsigned long long>(st.num_sol), [&] {
                  std::string s;
                  for (size_t i = 0; i < mac.solution.size(); ++i) s += (i ? ", " : "") + std::to_string(mac.solution[i]);
                  return s;
                }().c_str());
  }
  {
    Network net(engine, model);
    apply_init(net);
    GModel gm(&net);
    GModelSolver solver(&gm);
    GpuSearchStatistics st = solver.Solve(60000);
    std::vector<int> sol = solver.GetSolution();
    std::string s;
    for (size_t i = 0; i < sol.size(); ++i) s += (i ? ", " : "") + std::to_string(sol[i]);
    std::printf("{\"op\": \"gsolver\", \"num_solutions\": %d, \"unsolvable\": %s, \"solution\": [%s]}\n",
                st.num_solutions, st.unsolvable ? "true" : "false", s.c_str());
  }
  return 0;
}
