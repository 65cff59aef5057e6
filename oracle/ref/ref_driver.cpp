// Runs the reference's own CPU propagators on a seeded instance and prints the
// result as one JSON line. Test infrastructure: built by oracle/ref/Makefile
// against the reference sources where they lie (src/Network.cpp, src/AC3.cpp,
// src/AC3bit.cpp, src/SAC1.cpp, src/MAC.cpp, src/Solver.cpp, src/model/*.cpp)
// plus the absl/glog shim in oracle/shim. Its outputs pin the oracle
// restatement and become the golden fixtures under tests/golden/.
//
// Usage:
//   ref_driver binary N D E P_LO P_HI REMOVE SEED  OP [ARG]
//   ref_driver mixed  N D E P_LO P_HI K3 NTUP REMOVE SEED  OP [ARG]
//   ref_driver mixedbin (same arguments as mixed; tables dropped)
//   ref_driver uneven SEED N_LO N_HI D_CAP  OP [ARG]
//   ref_driver file PATH  OP [ARG]     (a binary network dumped as text:
//       "n W", n domain sizes, n*W initial words, "nb", nb scope pairs,
//       then every constraint's dom(x)*W support-row words, decimal)
// OP: ac3bit | ac3 | sac1 | mac | mac_domdeg | mac_domwdeg | time_ac REPS | time_branches K |
//     verdicts [FIRST [COUNT]]
#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>

#include "Network.h"
#include "Solver.h"
#include "model/model_builder.h"
#include "cp_gen.h"
#include "ref_model.h"

using namespace cpim;

using refmodel::apply_initial_domains;
using refmodel::build_model;

namespace {

std::string domains_hex(Network& net, const cpgen::Instance& I, int level) {
  std::string s;
  char buf[17];
  for (int x = 0; x < I.n; ++x) {
    auto& bd = net.vars[x]->bitDom(level);
    for (int w = 0; w < I.W; ++w) {
      const uint64_t v = w < int(bd.size()) ? bd[w].to_ullong() : 0ull;
      std::snprintf(buf, sizeof buf, "%016llx", static_cast<unsigned long long>(v));
      s += buf;
    }
  }
  return s;
}

struct Silence {
  std::streambuf* old;
  std::ofstream null;
  Silence() : null("/dev/null") { old = std::cout.rdbuf(null.rdbuf()); }
  ~Silence() { std::cout.rdbuf(old); }
};

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::cerr << "usage: see header" << std::endl;
    return 2;
  }
  std::string kind = argv[1];
  int i = 2;
  cpgen::Instance I;
  if (kind == "binary" && argc >= 10) {
    I = cpgen::random_binary(std::atoi(argv[2]), std::atoi(argv[3]), std::atoll(argv[4]), std::atof(argv[5]),
                             std::atof(argv[6]), std::atof(argv[7]), std::strtoull(argv[8], nullptr, 10));
    i = 9;
  } else if (kind == "mixed" && argc >= 12) {
    I = cpgen::random_mixed(std::atoi(argv[2]), std::atoi(argv[3]), std::atoll(argv[4]), std::atof(argv[5]),
                            std::atof(argv[6]), std::atoi(argv[7]), std::atoi(argv[8]), std::atof(argv[9]),
                            std::strtoull(argv[10], nullptr, 10));
    i = 11;
  } else if (kind == "mixedbin" && argc >= 12) {
    // The binary sub-network of a mixed instance: same binary constraints and
    // initial domains, tables dropped.
    I = cpgen::random_mixed(std::atoi(argv[2]), std::atoi(argv[3]), std::atoll(argv[4]), std::atof(argv[5]),
                            std::atof(argv[6]), std::atoi(argv[7]), std::atoi(argv[8]), std::atof(argv[9]),
                            std::strtoull(argv[10], nullptr, 10));
    I.tarity.clear();
    I.tscope_off.clear();
    I.tscope.clear();
    I.tntup.clear();
    I.ttup_off.clear();
    I.ttup.clear();
    i = 11;
  } else if (kind == "file" && argc >= 4) {
    // A dumped network (for instances read elsewhere, e.g. from XCSP files).
    std::ifstream in(argv[2]);
    if (!in) {
      std::cerr << "cannot open " << argv[2] << std::endl;
      return 2;
    }
    in >> I.n >> I.W;
    I.dom.resize(I.n);
    for (auto& d : I.dom) in >> d;
    I.init.resize(size_t(I.n) * I.W);
    for (auto& w : I.init) in >> w;
    int nb = 0;
    in >> nb;
    I.bx.resize(nb);
    I.by.resize(nb);
    for (int c = 0; c < nb; ++c) in >> I.bx[c] >> I.by[c];
    I.brow_off.resize(nb);
    for (int c = 0; c < nb; ++c) {
      I.brow_off[c] = int64_t(I.brows.size());
      for (int64_t k = 0; k < int64_t(I.dom[I.bx[c]]) * I.W; ++k) {
        uint64_t w = 0;
        in >> w;
        I.brows.push_back(w);
      }
    }
    if (!in) {
      std::cerr << "truncated network file" << std::endl;
      return 2;
    }
    // Optional positive tables: "nt", then per table its arity, scope,
    // tuple count and tuples.
    int nt = 0;
    if (in >> nt) {
      for (int t = 0; t < nt; ++t) {
        int r = 0, k = 0;
        in >> r;
        I.tarity.push_back(r);
        I.tscope_off.push_back(int64_t(I.tscope.size()));
        for (int q = 0; q < r; ++q) {
          int v = 0;
          in >> v;
          I.tscope.push_back(v);
        }
        in >> k;
        I.tntup.push_back(k);
        I.ttup_off.push_back(int64_t(I.ttup.size()));
        for (int64_t q = 0; q < int64_t(k) * r; ++q) {
          int v = 0;
          in >> v;
          I.ttup.push_back(v);
        }
      }
      if (!in) {
        std::cerr << "truncated table section" << std::endl;
        return 2;
      }
    }
    i = 3;
  } else if (kind == "uneven" && argc >= 7) {
    I = cpgen::uneven_instance(std::strtoull(argv[2], nullptr, 10), std::atoi(argv[3]), std::atoi(argv[4]),
                               std::atoi(argv[5]));
    i = 6;
  } else {
    std::cerr << "bad arguments" << std::endl;
    return 2;
  }
  const std::string op = argv[i];
  const long arg = (i + 1 < argc) ? std::atol(argv[i + 1]) : 0;

  model::IntermediateModel m = build_model(I);
  Network net(m);
  apply_initial_domains(net, I);

  std::ostringstream out;
  char fp[32];
  std::snprintf(fp, sizeof fp, "%016llx", static_cast<unsigned long long>(cpgen::fingerprint(I)));
  out << "{\"fingerprint\": \"" << fp << "\", \"n\": " << I.n << ", \"W\": " << I.W;

  if (op == "ac3bit" || op == "ac3") {
    AC* ac = (op == "ac3bit") ? static_cast<AC*>(new AC3bit(&net)) : static_cast<AC*>(new AC3(&net));
    ConsistencyState cs;
    {
      Silence s;
      cs = ac->enforce(net.vars, 0);
    }
    out << ", \"consistent\": " << (cs.state ? "true" : "false") << ", \"deletions\": " << cs.num_delete;
    if (cs.state) out << ", \"domains\": \"" << domains_hex(net, I, 0) << "\"";
    delete ac;
  } else if (op == "sac1" || op == "sac1_ac3") {
    // sac1_ac3: SAC1 over the generic AC3 (tables of any arity).
    SAC1 sac(&net, op == "sac1" ? AC_3bit : AC_3);
    bool ok;
    {
      Silence s;
      ok = sac.enforce(net.vars, 0);
    }
    out << ", \"consistent\": " << (ok ? "true" : "false") << ", \"deletions\": " << sac.del();
    if (ok) out << ", \"domains\": \"" << domains_hex(net, I, 0) << "\"";
  } else if (op == "mac" || op == "mac_domdeg" || op == "mac_domwdeg" || op == "mac_ac3" || op == "mac_ac3_domdeg") {
    // mac_ac3*: MAC over the generic AC3 (tables of any arity).
    const Heuristic::Var vh = (op == "mac" || op == "mac_ac3") ? Heuristic::VRH_DOM_MIN
                              : (op == "mac_domdeg" || op == "mac_ac3_domdeg") ? Heuristic::VRH_DOM_DEG_MIN
                                                                               : Heuristic::VRH_DOM_WDEG_MIN;
    const bool generic = op == "mac_ac3" || op == "mac_ac3_domdeg";
    MAC mac(&net, generic ? AC_3 : AC_3bit, vh, Heuristic::VLH_MIN);
    SearchStatistics st;
    const double t0 = now_s();
    {
      Silence s;
      st = mac.enforce(arg > 0 ? int(arg) : 600000);
    }
    const double t1 = now_s();
    out << ", \"num_positive\": " << st.num_positive << ", \"num_negative\": " << st.num_negative
        << ", \"num_sol\": " << st.num_sol << ", \"time_out\": " << (st.time_out ? "true" : "false")
        << ", \"solve_ms\": " << (t1 - t0) * 1e3
        << ", \"solution\": [";
    for (size_t k = 0; k < mac.solution.size(); ++k) out << (k ? ", " : "") << mac.solution[k];
    out << "]";
  } else if (op == "time_ac") {
    const int reps = arg > 0 ? int(arg) : 3;
    AC3bit ac(&net);
    double best = 1e30;
    int dels = 0;
    bool ok = true;
    for (int r = 0; r < reps; ++r) {
      net.CopyLevel(0, 1);
      const double t0 = now_s();
      auto cs = ac.enforce(net.vars, 1);
      const double t1 = now_s();
      best = std::min(best, t1 - t0);
      dels = cs.num_delete;
      ok = cs.state;
    }
    out << ", \"consistent\": " << (ok ? "true" : "false") << ", \"deletions\": " << dels
        << ", \"best_s\": " << best;
  } else if (op == "time_branches") {
    // The singleton test of SAC1::enforce (src/SAC1.cpp:70-79) on the first K
    // live (x, a), timed; no deletion is committed.
    const long K = arg > 0 ? arg : 100;
    AC3bit ac(&net);
    std::vector<IntVar*> evt;
    long done = 0, failed = 0;
    const double t0 = now_s();
    for (auto* x : net.vars) {
      for (int a : x->values()) {
        if (done >= K) break;
        if (!x->have(a, 0)) continue;
        net.CopyLevel(0, net.tmp());
        x->ReduceTo(a, net.tmp());
        x->assign(true, net.tmp());
        evt.push_back(x);
        failed += ac.enforce(evt, net.tmp()).state ? 0 : 1;
        evt.clear();
        x->assign(false, 0);
        net.ClearLevel(net.tmp());
        ++done;
      }
      if (done >= K) break;
    }
    const double t1 = now_s();
    out << ", \"branches\": " << done << ", \"failed\": " << failed << ", \"seconds\": " << (t1 - t0);
  } else if (op == "verdicts") {
    // Root AC3bit, then the singleton test of SAC1::enforce (src/SAC1.cpp:
    // 70-79) on every live (x, a) of the closure, in the reference's loop
    // order, all against the same root domains (nothing is removed). Live
    // pairs FIRST .. FIRST+COUNT-1 of that order are tested (all by default),
    // so callers can split the work over processes. Prints the failed pairs.
    const long first = arg;
    const long count = (i + 2 < argc) ? std::atol(argv[i + 2]) : -1;
    AC3bit ac(&net);
    ConsistencyState cs;
    {
      Silence s;
      cs = ac.enforce(net.vars, 0);
    }
    out << ", \"consistent\": " << (cs.state ? "true" : "false");
    if (cs.state) {
      std::vector<IntVar*> evt;
      long idx = 0, tested = 0;
      out << ", \"failed\": [";
      bool firstf = true;
      for (auto* x : net.vars) {
        for (int a : x->values()) {
          if (!x->have(a, 0)) continue;
          const long k = idx++;
          if (k < first || (count >= 0 && k >= first + count)) continue;
          net.CopyLevel(0, net.tmp());
          x->ReduceTo(a, net.tmp());
          x->assign(true, net.tmp());
          evt.push_back(x);
          bool res;
          {
            Silence s;
            res = ac.enforce(evt, net.tmp()).state;
          }
          evt.clear();
          x->assign(false, 0);
          net.ClearLevel(net.tmp());
          ++tested;
          if (!res) {
            out << (firstf ? "" : ", ") << "[" << x->id() << ", " << a << "]";
            firstf = false;
          }
        }
      }
      out << "], \"live\": " << idx << ", \"tested\": " << tested;
    }
  } else {
    std::cerr << "unknown op " << op << std::endl;
    return 2;
  }
  out << "}";
  std::cout << out.str() << std::endl;
  return 0;
}
