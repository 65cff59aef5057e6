// Builds the reference's own Network (its sources, compiled by
// oracle/ref/Makefile) for a seeded instance twice and runs the same
// propagation through the reference's AC3bit and through GpuAC
// (include/gpu_ac.hpp, the adapter a maintainer adds to the reference):
// the root AC at level 0, then the singleton test of SAC1::enforce
// (src/SAC1.cpp:70-79) for the first PROBES live values, each on the tmp
// level. Prints one JSON object: verdicts and domains compared.
//
// Usage: gpu_ac_check N D E P REMOVE SEED PROBES
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "Network.h"
#include "Solver.h"
#include "cp_gen.h"
#include "gpu_ac.hpp"
#include "ref_model.h"

using namespace cpim;

static bool same_level(Network& a, Network& b, int level) {
  for (size_t x = 0; x < a.vars.size(); ++x)
    if (a.vars[x]->bitDom(level) != b.vars[x]->bitDom(level)) return false;
  return true;
}

int main(int argc, char** argv) {
  if (argc < 8) {
    std::fprintf(stderr, "usage: gpu_ac_check N D E P REMOVE SEED PROBES\n");
    return 2;
  }
  const cpgen::Instance I =
      cpgen::random_binary(std::atoi(argv[1]), std::atoi(argv[2]), std::atoll(argv[3]), std::atof(argv[4]),
                           std::atof(argv[4]), std::atof(argv[5]), std::strtoull(argv[6], nullptr, 10));
  const long probes = std::atol(argv[7]);
  model::IntermediateModel m = refmodel::build_model(I);
  Network ref(m), gpu(m);
  refmodel::apply_initial_domains(ref, I);
  refmodel::apply_initial_domains(gpu, I);
  AC3bit ac_ref(&ref);
  GpuAC ac_gpu(&gpu);
  ConsistencyState a = ac_ref.enforce(ref.vars, 0);
  ConsistencyState b = ac_gpu.enforce(gpu.vars, 0);
  const bool root_same = a.state == b.state && (!a.state || (same_level(ref, gpu, 0) && a.num_delete == b.num_delete));
  long tested = 0, mismatches = 0, failed = 0;
  if (a.state && b.state) {
    std::vector<IntVar*> evt_ref, evt_gpu;
    for (size_t xi = 0; xi < ref.vars.size() && tested < probes; ++xi) {
      IntVar* xr = ref.vars[xi];
      IntVar* xg = gpu.vars[xi];
      for (int v : xr->values()) {
        if (tested >= probes) break;
        if (!xr->have(v, 0)) continue;
        ref.CopyLevel(0, ref.tmp());
        gpu.CopyLevel(0, gpu.tmp());
        xr->ReduceTo(v, ref.tmp());
        xg->ReduceTo(v, gpu.tmp());
        xr->assign(true, ref.tmp());
        xg->assign(true, gpu.tmp());
        evt_ref.assign(1, xr);
        evt_gpu.assign(1, xg);
        const bool r = ac_ref.enforce(evt_ref, ref.tmp()).state;
        const bool g = ac_gpu.enforce(evt_gpu, gpu.tmp()).state;
        if (r != g || (r && !same_level(ref, gpu, ref.tmp()))) ++mismatches;
        failed += r ? 0 : 1;
        xr->assign(false, 0);
        xg->assign(false, 0);
        ref.ClearLevel(ref.tmp());
        gpu.ClearLevel(gpu.tmp());
        ++tested;
      }
    }
  }
  std::printf("{\"consistent\": %s, \"root_same\": %s, \"probes\": %ld, \"failed\": %ld, \"mismatches\": %ld}\n",
              a.state ? "true" : "false", root_same ? "true" : "false", tested, failed, mismatches);
  return root_same && mismatches == 0 ? 0 : 1;
}
