"""Benchmark: batched SAC1 sweep on one GB300 (SAC fixpoints/s).

Workload (one step): the SAC closure of a model-B random binary network with
n=500 variables, uniform domains of d=128 values (two u64 words), e=10000
constraints on distinct random pairs, tightness p=0.40, seed 7 -- root AC,
then every live (x, a) singleton test (n*d = 64000 branch fixpoints) in one
persistent launch per sweep, until no test fails. Synthetic inputs with the
shape of the published workload; generated by cpim_gb300/csrc/cp_gen.h.

A step is a batch of R such closures (R = --closures-per-step, default 128),
so that even a short run (--steps 20) keeps the GPU busy for over a second
and the clock sampler sees it. value: singleton fixpoints per second over K
steps, inputs resident in HBM, CUDA-event device time of each enforce call;
L2 is flushed (a 256 MiB write) before every closure. e2e: the same metric
through the C ABI with host buffers: every closure re-uploads the relations
and domains from pinned host memory, runs cp_enforce_sac1 and reads the final
domains back; two engines alternate, so that closure i+1's upload
(cp_net_reload_async) overlaps closure i, whose domains come back with
cp_enforce_sac1_end_domains (e2e.sequential_value: the same without the
overlap, cp_net_reload, cp_enforce_sac1 and cp_dom_get).

Outside the timed region the line also carries: parity (every first-sweep
singleton verdict and the SAC closure against the oracle on the host cores),
the roofline of the sweep kernels (with and without the per-branch domain
copy term, and the DRAM fraction from the committed ncu capture in
profiles/k_sac_tile_cfg3_sweep.json), the large GAC fixpoint, and a
256-instance sample of the uneven batch against its one-by-one rate.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, D, E, P, SEED = 500, 128, 10000, 0.40, 7
WORKLOAD = "batched SAC1 sweep: model-B binary CSP n=500 d=128 e=10000 p=0.40 seed=7 (n*d=64000 singleton branches)"
METRIC = "SAC fixpoints/s (batched singleton AC closures, bit-exact)"
UNIT = "fixpoints/s"


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def sweep_profile():
    """The committed ncu figures of the SAC sweep kernels on this workload
    (profiles/k_sac_tile_cfg3_sweep.json: DRAM bytes per sweep, limiter), or
    an empty dict."""
    try:
        with open(os.path.join(ROOT, "profiles", "k_sac_tile_cfg3_sweep.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def bench_config(**extra):
    """The config dict both arms print."""
    c = {"workload": WORKLOAD, "n": N, "d": D, "e": E, "p": P, "seed": SEED}
    c.update(extra)
    return c


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def oracle_instance():
    """The benchmark network from the oracle library's copy of the generator
    (the same cp_gen.h the engine compiles; fingerprints are compared)."""
    from oracle import pyoracle as O
    return O.gen_binary(N, D, E, P, P, 0.0, SEED)


def cpu_baseline_port(ov, threads, budget_s=15.0):
    """The oracle's SAC singleton test (the reference's AC3bit inner loop,
    restated) on host cores over an evenly spread sample of branches."""
    from oracle import pyoracle as O
    s1, done1, _ = O.time_singletons(ov, ov.init, 64, 1)
    per_branch = s1 / max(1, done1)
    count = int(max(256, min(64000, budget_s / per_branch)))
    secs, done, failed = O.time_singletons(ov, ov.init, count, threads)
    return {"value": done / secs, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d of the %d singleton branches (evenly spread), oracle AC3bit restatement, %d host threads"
                      % (done, N * D, threads),
            "seconds": secs, "single_thread_ms_per_branch": per_branch * 1e3}


def run_reference(args):
    """The reference's CPU singleton test (its restatement in oracle/; the
    reference's own build does not travel to this host) on all host threads.
    Loads only the oracle library: the engine is not imported."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import pyoracle
    pyoracle.build()
    inst = oracle_instance()
    threads = os.cpu_count() or 1
    vals = []
    # Each step is a bounded sample sized so the whole run stays near 90 s of
    # wall time on the host's cores.
    per_step_wall = max(0.05, 90.0 / max(1, args.warmup + args.steps))
    for i in range(args.warmup + args.steps):
        r = cpu_baseline_port(inst, threads, budget_s=per_step_wall * threads)
        if i >= args.warmup:
            vals.append(r["value"])
    v = statistics.median(vals)
    base = cpu_baseline_port(inst, threads, budget_s=2.0 * threads)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded generator)",
            "config": bench_config(), "parallelism": "host threads (%d)" % threads,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": base["sample"] + "; per step, median over steps"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference's CPU path compiles only in the build container (x86, sources present); "
                    "on this host its restatement in oracle/ is timed"}
    print(json.dumps(line))
    return 0


def parity_check(net, final, eng_fp):
    """Outside the timed region: one Jacobi sweep of singleton tests through
    the sweep kernels (cp_sac_sweep) against the oracle's verdicts for every
    live (x, a), and the timed closure against the oracle's SAC closure, both
    on all host threads."""
    import numpy as np
    from oracle import pyoracle as O
    ov = oracle_instance()
    assert ov.fingerprint == eng_fp, "engine and oracle generators disagree"
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ok_ac, d_ac, _ = O.ac3bit(ov)
    ver_o, failed_o = O.singleton_verdicts(ov, d_ac, threads)
    ok_s, d_sac, _, sweeps_o = O.sac_jacobi(ov, None, threads)
    oracle_s = time.perf_counter() - t0
    net.dom_set(0, ov.init)
    ver_g, deep, st = net.sac_sweep(0)
    live = int(sum(bin(int(w)).count("1") for w in d_ac))
    diff = int(sum(bin(int(a) ^ int(b)).count("1") for a, b in zip(ver_g, ver_o)))
    return {"first_sweep_verdicts": {"live_values": live, "equal": live - diff, "failed_oracle": failed_o,
                                     "deep_list": int(deep), "bit_exact": diff == 0},
            "closure": {"bit_exact": bool(ok_s and np.array_equal(final, d_sac)), "oracle_sweeps": sweeps_o},
            "oracle": "oracle/ restatement of AC3bit + SAC1 singleton tests, %d host threads, %.1f s"
                      % (threads, oracle_s)}


def tensor_variant(inst, net, sweep_ms, reps=3):
    """The support-count formulation of round two on the tensor cores against
    the bitwise test, on the same tiles of the benchmark network: every (x, y,
    z) tile of the first variables (128 branches x = a, K = 128 values of y,
    N = 128 values of z), outputs compared bit for bit. A full sweep needs one
    such tile per (x, y, z) path; both costs are projected to that count and
    set beside the measured sweep kernels (which skip nearly all of it)."""
    import numpy as np
    import cpim_gb300 as cp
    tx, t1, t2 = cp.sac_tile_list(inst, range(N), limit=16384)
    res = {}
    outs = {}
    for mode, name in ((0, "bitwise"), (1, "tensor_cores")):
        best = 1e30
        for _ in range(reps):
            out, ms = net.sac_tiles(tx, t1, t2, mode=mode)
            best = min(best, ms)
        outs[mode] = out
        res[name] = {"ms": best, "tiles_per_s": len(tx) / (best / 1e3)}
    assert np.array_equal(outs[0], outs[1])
    deg = np.bincount(inst.bin_scope, minlength=inst.n)
    bx, by = inst.bin_scope[0::2], inst.bin_scope[1::2]
    sweep_tiles = int(((deg[bx] - 1) + (deg[by] - 1)).sum())
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16 = float(json.load(f)["bf16_tflops"])
    except Exception:
        bf16 = 1900.0
    flops = 2.0 * 128 ** 3 * len(tx)
    tc = res["tensor_cores"]
    tc["tflops"] = flops / (tc["ms"] / 1e3) / 1e12
    tc["frac_of_bf16_peak"] = tc["tflops"] / bf16
    for name in res:
        res[name]["projected_sweep_ms"] = sweep_tiles / res[name]["tiles_per_s"] * 1e3
    return {"tiles": len(tx), "tile_shape": "M=128 branches x K=128 values of y x N=128 values of z",
            "outputs_equal": True, "sweep_tiles": sweep_tiles, "measured_sweep_kernels_ms": sweep_ms,
            "bf16_peak_tflops": bf16, **res,
            "kept": "bitwise (the tensor form cannot skip arcs with the weak-support bound)"}


def gac_sample(eng, peak, flush, steps=20, warmup=3):
    """The large GAC fixpoint (n=2000, d=64, 30000 binary + 5000 ternary
    tables with 500 tuples, 20% of values removed, seed 1) on the grid-wide
    kernel: median CUDA-event time over `steps` runs, L2 flushed before each,
    verdict checked against the oracle."""
    import torch
    import cpim_gb300 as cp
    from oracle import pyoracle as O
    inst = cp.gen_mixed(2000, 64, 30000, 0.2, 0.5, 5000, 500, 0.2, 1)
    net = eng.upload(inst, max_levels=2)
    sts = []
    for i in range(warmup + steps):
        net.dom_set(0, inst.init)
        flush.fill_(1)
        torch.cuda.synchronize()
        st = net.enforce_ac(0)
        if i >= warmup:
            sts.append(st)
    ms = statistics.median(s.device_ms for s in sts)
    st = sts[-1]
    ok, _, dels = O.gac(O.Instance(n=inst.n, W=inst.W, dom=inst.dom, init=inst.init,
                                   bx=inst.bin_scope[0::2].copy(), by=inst.bin_scope[1::2].copy(),
                                   brows=inst.bin_rows, tarity=inst.tab_arity, tscope=inst.tab_scope,
                                   tntup=inst.tab_ntup, ttup=inst.tab_tuples))
    net.close()
    ach = st.alg_bytes / (ms / 1e3) / 1e9
    return {"workload": "GAC fixpoint: n=2000 d=64, 30000 binary (p~U[0.2,0.5]) + 5000 ternary positive tables "
                        "(500 tuples), 20% of values removed, seed 1; L2 flushed before each run",
            "ms": ms, "revisions_per_s": st.revisions / (ms / 1e3), "rounds": int(st.rounds),
            "inconsistent": bool(st.inconsistent), "verdict_equals_oracle": ok == (not st.inconsistent),
            "alg_gb_per_s": ach, "frac_of_hbm_peak": ach / peak}


def uneven_sample(eng, k=256, per_instance=64):
    """A k-instance sample of the uneven batch (seeds 7*1000003+i): AC + SAC1
    of every member in one batch (graph-replayed sweeps, tuned), against the
    first `per_instance` members run one by one."""
    import cpim_gb300 as cp
    nets = []
    for i in range(k):
        net = cp.upload_uneven_device(eng, 7 * 1000003 + i, 20, 400, 256, max_levels=2)
        net.level_copy(0, 1)
        nets.append(net)
    batch = cp.Batch(eng, nets, level=0)
    batch.tune()
    ms = []
    for _ in range(3):
        batch.copy_level(1)
        st, inc = batch.sac1()
        ms.append(st.device_ms)
    batch.close()
    t = 0.0
    for net in nets[:per_instance]:
        net.level_copy(1, 0)
        t += net.enforce_sac1(0).device_ms
    sub = cp.Batch(eng, nets[:per_instance], level=0)
    sub_ms = []
    for _ in range(2):
        sub.copy_level(1)
        sub_ms.append(sub.sac1()[0].device_ms)
    sub.close()
    for n in nets:
        n.close()
    one = per_instance / (t / 1e3)
    same = per_instance / (min(sub_ms) / 1e3)
    return {"workload": UNEVEN_WORKLOAD.format(k=k), "instances_per_s": k / (min(ms) / 1e3),
            "ms_per_batch": min(ms), "inconsistent_instances": int(inc.sum()),
            "one_by_one": {"instances": per_instance, "instances_per_s": one,
                           "batched_same_instances_per_s": same, "batched_over_one_by_one": same / one}}


def run_ours(args):
    import numpy as np
    import torch
    import cpim_gb300 as cp

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    R = args.closures_per_step
    inst = cp.gen_binary(N, D, E, P, P, 0.0, SEED)
    eng = cp.Engine(local)
    # High stream priority: the e2e leg's overlapped reloads (lowest priority)
    # then take SMs only where the closures leave them free.
    eng.set_priority(1)
    net = eng.upload(inst, max_levels=2)
    pristine = inst.init.copy()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def closure():
        net.dom_set(0, pristine)
        flush.fill_(1)
        torch.cuda.synchronize()
        return net.enforce_sac1(0)

    def step():
        return [closure() for _ in range(R)]

    for _ in range(args.warmup):
        step()
    barrier()
    torch.cuda.synchronize()
    launches0 = eng.launches
    sts = []
    if args.quick:
        # Profiling mode: the timed steps only, no baselines and no e2e leg.
        for _ in range(args.steps):
            sts += step()
        torch.cuda.synchronize()
        if rank == 0:
            print(json.dumps({"quick": True, "closures": len(sts),
                              "ms_per_closure": sum(s.device_ms for s in sts) / len(sts),
                              "kernel_ms": sum(s.kernel_ms for s in sts) / len(sts),
                              "branches": int(sts[-1].branches)}))
        return 0
    t_wall = time.perf_counter()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            sts += step()
        torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    barrier()
    gpu_launches = eng.launches - launches0
    dev_ms = [s.device_ms for s in sts]
    branches = sum(s.branches for s in sts)
    # Replicas: branches summed over ranks, the slowest rank's device time.
    from cpim_gb300.replicas import job_rate
    _, job_s, value = job_rate(branches, sum(dev_ms) / 1e3, device="cuda")
    total_ms = job_s * 1e3
    final = net.dom_get(0)
    assert not sts[-1].inconsistent

    # Roofline of the dominant kernels: the sweep kernels of each closure.
    kern_ms = sum(s.kernel_ms for s in sts)
    kern_bytes = sum(s.kernel_bytes for s in sts)
    launches_k = sum(s.sweeps for s in sts)
    copy_bytes = float(branches) * 2 * N * inst.W * 8
    peak, peak_kind = measured_peaks()
    achieved = (kern_bytes / (kern_ms / 1e3)) / 1e9 if kern_ms > 0 else 0.0
    achieved_nc = ((kern_bytes - copy_bytes) / (kern_ms / 1e3)) / 1e9 if kern_ms > 0 else 0.0
    prof = sweep_profile()
    traffic = prof.get("dram_bytes_per_sweep")
    kms_launch = kern_ms / max(1, launches_k)
    dram_gbs = traffic / (kms_launch / 1e3) / 1e9 if traffic else None

    # e2e through the C ABI with pinned host buffers.
    rows_pin = torch.from_numpy(inst.bin_rows.view(np.int64)).pin_memory()
    init_pin = torch.from_numpy(inst.init.view(np.int64)).pin_memory()
    rows_np = rows_pin.numpy().view(np.uint64)
    init_np = init_pin.numpy().view(np.uint64)
    e2e_inst = cp.Instance(n=inst.n, W=inst.W, dom=inst.dom, init=init_np, bin_scope=inst.bin_scope,
                           bin_rows=rows_np, tab_arity=inst.tab_arity, tab_scope=inst.tab_scope,
                           tab_ntup=inst.tab_ntup, tab_tuples=inst.tab_tuples)
    out = np.zeros(inst.n * inst.W, np.uint64)

    parts = {"reload": [], "enforce": [], "dom_get": []}

    def e2e_closure():
        t0 = time.perf_counter()
        net.reload(e2e_inst)
        t1 = time.perf_counter()
        st = net.enforce_sac1(0)
        t2 = time.perf_counter()
        r = net.dom_get(0)
        t3 = time.perf_counter()
        parts["reload"].append(t1 - t0)
        parts["enforce"].append(t2 - t1)
        parts["dom_get"].append(t3 - t2)
        return st, r

    # Pipelined: two engines, one copy of the network each; while one engine
    # runs closure i (cp_enforce_sac1_begin / _end), closure i+1's relations
    # and domains go to the other (cp_net_reload_async, on that engine's
    # lowest-priority transfer stream).
    # Every closure still uploads its inputs from pinned host memory and
    # reads its domains back.
    eng_b = cp.Engine(local)
    eng_b.set_priority(1)
    net_b = eng_b.upload(inst, max_levels=2)
    pair = (net, net_b)

    def e2e_pipelined(count):
        pair[0].reload_async(e2e_inst)
        br, r = 0, None
        for i in range(count):
            cur = pair[i % 2]
            cur.enforce_sac1_begin(0)  # queued behind its own reload
            if i + 1 < count:
                pair[(i + 1) % 2].reload_async(e2e_inst)
            st, r = cur.enforce_sac1_end_domains()  # the closure comes back with the call
            assert np.array_equal(r, final)
            br += st.branches
        return br, r

    for _ in range(max(1, args.warmup)):
        e2e_closure()
        e2e_pipelined(2)
    torch.cuda.synchronize()
    e2e_steps = max(1, args.steps // 4)
    t0 = time.perf_counter()
    e2e_seq_br = 0
    for _ in range(e2e_steps * R):
        st, r = e2e_closure()
        e2e_seq_br += st.branches
    torch.cuda.synchronize()
    e2e_seq_s = time.perf_counter() - t0
    assert np.array_equal(r, final)
    _, _, e2e_seq_value = job_rate(e2e_seq_br, e2e_seq_s, device="cuda")
    t0 = time.perf_counter()
    e2e_br, r = e2e_pipelined(e2e_steps * R)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    _, _, e2e_value = job_rate(e2e_br, e2e_s, device="cuda")
    # What bounds it: the host-to-device bandwidth of the relation rows
    # (torch copy of the same pinned buffer) and the per-call wall times of
    # the sequential leg.
    dev_rows = torch.empty(rows_pin.numel(), dtype=torch.int64, device="cuda")
    h2d = []
    for _ in range(10):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev_rows.copy_(rows_pin, non_blocking=True)
        torch.cuda.synchronize()
        h2d.append(time.perf_counter() - t0)
    e2e_parts = {k + "_us": 1e6 * float(np.median(v)) for k, v in parts.items()}
    e2e_parts["h2d_rows_gb_per_s"] = rows_pin.numel() * 8 / float(np.median(h2d)) / 1e9
    del dev_rows

    # Plain single-instance path: one launch per singleton test (sample).
    rng = np.random.default_rng(1)
    k = 2000
    xs = rng.integers(0, N, k).astype(np.int32)
    vs = rng.integers(0, D, k).astype(np.int32)
    net.dom_set(0, pristine)
    net.singletons(xs[:100], vs[:100], mode=1)
    ok_p, st_p = net.singletons(xs, vs, mode=1)
    ok_b, st_b = net.singletons(xs, vs, mode=0)
    assert np.array_equal(ok_p, ok_b)
    plain_rate = k / (st_p.device_ms / 1e3)

    if rank != 0:
        return 0
    clocks = clk.summary()
    parity = parity_check(net, final, inst.fingerprint)
    net.dom_set(0, pristine)
    tensor = tensor_variant(inst, net, kms_launch)
    gac = gac_sample(eng, peak, flush) if not args.no_extras else None
    uneven = uneven_sample(eng) if not args.no_extras else None
    base = cpu_baseline_port(oracle_instance(), os.cpu_count() or 1)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded generator, shape of the published workload)",
        "config": bench_config(),
        "step": "%d SAC closures of the network (each %d branch fixpoints over %d sweep(s)), L2 flushed "
                "(256 MiB write) and the domains reset before each closure" % (R, int(sts[-1].branches),
                                                                                int(sts[-1].sweeps)),
        "parallelism": "replicas (%d GPUs)" % world if world > 1 else "single GPU",
        "timed_wall_s": t_wall,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(R * (inst.bin_rows.nbytes + inst.init.nbytes)),
                "d2h_bytes_per_step": int(R * out.nbytes), "steps": e2e_steps,
                "mode": "each closure's upload overlapped with the previous closure on a second engine "
                        "(cp_net_reload_async); the closure's domains returned by cp_enforce_sac1_end_domains",
                "sequential_value": e2e_seq_value, "sequential_median_per_call": e2e_parts},
        "gpu_launches": int(gpu_launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "frac_without_branch_copy": achieved_nc / peak,
                     "dram_frac": (dram_gbs / peak) if dram_gbs else None,
                     "kernel": "SAC sweep kernels (k_work_and_weak + k_sac_tile + k_sac on the deep list), per sweep",
                     "kernel_ms_per_launch": kms_launch,
                     "alg_bytes_per_launch": kern_bytes / max(1, launches_k),
                     "branch_copy_bytes_per_launch": copy_bytes / max(1, launches_k),
                     "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic_source": prof.get("source"), "limiter": prof.get("limiter")},
        "parity": parity,
        "cpu_baseline": {k2: base[k2] for k2 in ("value", "unit", "cores", "kind", "sample")},
        "plain_single_instance": {"value": plain_rate, "unit": UNIT,
                                  "sample": "%d singleton tests, one single-CTA launch each" % k,
                                  "batched_over_plain": value / plain_rate},
        "tensor_variant": tensor,
        "gac_large": gac,
        "uneven_sample": uneven,
        "clocks": clocks,
    }
    print(json.dumps(line))
    net.close()
    eng.close()
    return 0


UNEVEN_WORKLOAD = ("uneven multi-instance batch: {k} random binary CSPs, n~U[20,400], d in {{8..256}}, "
                   "density~U[0.05,0.3], tightness~U[0.2,0.6], seeds 7*1000003+i; AC + SAC1 of every instance")


def run_uneven(args):
    """Config-4 measurement: AC + SAC1 of every instance of the uneven batch in
    one launch per phase (graph-replayed sweeps), against the same instances
    run one by one through cp_enforce_sac1."""
    import torch
    import cpim_gb300 as cp

    torch.cuda.set_device(0)
    K = args.instances
    eng = cp.Engine(0)
    t0 = time.time()
    nets = []
    for i in range(K):
        net = cp.upload_uneven_device(eng, 7 * 1000003 + i, 20, 400, 256, max_levels=2)
        net.level_copy(0, 1)
        nets.append(net)
    gen_s = time.time() - t0
    dev_bytes = sum(n.device_bytes for n in nets)
    batch = cp.Batch(eng, nets, level=0)
    batch.tune()
    launches0 = eng.launches

    def step():
        batch.copy_level(1)
        return batch.sac1()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches0 = eng.launches
    sts = []
    with ClockSampler(0) as clk:
        for _ in range(args.steps):
            sts.append(step())
    torch.cuda.synchronize()
    gpu_launches = eng.launches - launches0
    ms = [s.device_ms for s, _ in sts]
    st, inc = sts[-1]
    inst_rate = K / (statistics.median(ms) / 1e3)
    branch_rate = st.branches / (statistics.median(ms) / 1e3)
    # One instance at a time through the single-instance entry point, against
    # a batch of the same M instances.
    M = min(K, args.per_instance_sample)
    t_dev = 0.0
    t0 = time.perf_counter()
    for net in nets[:M]:
        net.level_copy(1, 0)
        t_dev += net.enforce_sac1(0).device_ms
    t_wall = time.perf_counter() - t0
    per_inst = M / (t_dev / 1e3)
    per_inst_wall = M / t_wall
    sub = cp.Batch(eng, nets[:M], level=0)
    sub_ms = []
    for _ in range(2):
        sub.copy_level(1)
        t1 = time.perf_counter()
        s_st, _ = sub.sac1()
        sub_ms.append(s_st.device_ms)
    sub.close()
    sub_rate = M / (min(sub_ms) / 1e3)

    # The same comparison on the smallest members (n*d <= 2048), where one
    # instance alone leaves most of the GPU idle.
    shapes = [cp._uneven_shape(7 * 1000003 + i, 20, 400, 256) for i in range(K)]
    small = [i for i in range(K) if shapes[i][0] * shapes[i][1] <= 2048][:M]

    def one_by_one(idx):
        t = 0.0
        for i in idx:
            nets[i].level_copy(1, 0)
            t += nets[i].enforce_sac1(0).device_ms
        return len(idx) / (t / 1e3)

    def batched(idx):
        b2 = cp.Batch(eng, [nets[i] for i in idx], level=0)
        best = 1e30
        for _ in range(2):
            b2.copy_level(1)
            best = min(best, b2.sac1()[0].device_ms)
        b2.close()
        return len(idx) / (best / 1e3)

    small_cmp = None
    if small:
        a, b_ = one_by_one(small), batched(small)
        small_cmp = {"instances": len(small), "value_device": a, "batched_same_instances": b_,
                     "batched_over_per_instance": b_ / a, "unit": "instances/s"}
    line = {"metric": "instance AC+SAC fixpoints/s (uneven batch, bit-exact)", "value": inst_rate,
            "unit": "instances/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.median(ms), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded, relations generated on the device)",
            "config": {"workload": UNEVEN_WORKLOAD.format(k=K), "instances": K,
                       "device_bytes": dev_bytes, "generate_upload_s": gen_s,
                       "inconsistent_instances": int(inc.sum()), "sweeps": int(st.sweeps),
                       "groups": [batch.info(g) for g in range(batch.info(0)["groups"])]},
            "branch_fixpoints_per_s": branch_rate, "branches_per_step": int(st.branches),
            "per_instance_launches": {"instances": M, "value_device": per_inst, "value_wall": per_inst_wall,
                                      "unit": "instances/s", "batched_same_instances": sub_rate,
                                      "batched_over_per_instance": sub_rate / per_inst},
            "small_members_n_times_d_le_2048": small_cmp,
            "gpu_launches": int(gpu_launches), "clocks": clk.summary()}
    print(json.dumps(line))
    batch.close()
    for n in nets:
        n.close()
    eng.close()
    return 0


SERVING_WORKLOAD = ("serving: Poisson arrivals, requests propagate:SAC:MAC-solve = 70:20:10 on {r} resident networks "
                    "(random binary CSPs, n~U[20,400], d in {{8..128}}, density~U[0.05,0.3], tightness~U[0.2,0.6], "
                    "seeds 5*1000003+i), 0-3 random variable choices per request, HBM budget 150 GB")


def _serving_trace(rng, rate, k, ids, shapes):
    """k requests: Poisson arrivals at `rate`, types 70:20:10, a uniformly
    drawn resident network, 0-3 (var, value) choices."""
    import numpy as np
    types = rng.choice(3, size=k, p=[0.7, 0.2, 0.1])
    gaps = rng.exponential(1.0 / rate, size=k)
    arrivals = np.cumsum(gaps) - gaps[0]
    reqs = []
    for t in types:
        j = int(rng.integers(0, len(ids)))
        n, d = shapes[j]
        ch = [(int(rng.integers(0, n)), int(rng.integers(0, d))) for _ in range(int(rng.integers(0, 4)))]
        reqs.append((int(t), ids[j], ch))
    return arrivals, reqs, types


def run_serving(args):
    """Config-5 measurement: request latency and throughput of the server
    with continuous batching, beside the one-request-per-launch path."""
    import numpy as np
    import torch
    import cpim_gb300 as cp

    torch.cuda.set_device(0)
    R = args.networks
    seeds = [5 * 1000003 + i for i in range(R)]
    t0 = time.time()
    # Config 4's size distribution capped at config 3's shape (d <= 128).
    hs = [cp.InstanceHandle.uneven(sd, 20, 400, 128) for sd in seeds]
    shapes = [cp._uneven_shape(sd, 20, 400, 128) for sd in seeds]
    gen_s = time.time() - t0
    rates = [float(x) for x in args.rates.split(",")]
    modes = [("batched", True), ("plain", False)]
    results = {}
    launches = 0
    with ClockSampler(0) as clk:
        for mode, batching in modes:
            rng = np.random.default_rng(11)
            with cp.Server(budget_bytes=150 * 10**9, max_batch=args.max_batch, batching=batching,
                           solve_time_limit_ms=args.solve_limit_ms, solvers=args.solvers) as srv:
                t1 = time.time()
                ids = [srv.register(h, slots=args.slots) for h in hs]
                reg_s = time.time() - t1
                # Warm-up: pools, tuning cache, solver copies.
                arr, reqs, _ = _serving_trace(rng, 2000.0, 200, ids, shapes)
                srv.run_trace(arr, reqs)
                l0 = srv.eA.launches + srv.eB.launches
                pts = []
                for rate in rates:
                    k = int(min(args.requests, max(50, rate * args.duration)))
                    arr, reqs, types = _serving_trace(rng, rate, k, ids, shapes)
                    lat, st, stats = srv.run_trace(arr, reqs)
                    ok = st == 2
                    pt = {"offered_rps": rate, "requests": k, "completed": int(ok.sum()),
                          "errors": int((~ok).sum()), "wall_s": stats[2], "throughput_rps": k / stats[2],
                          "p50_ms": float(np.percentile(lat[ok], 50)) if ok.any() else None,
                          "p99_ms": float(np.percentile(lat[ok], 99)) if ok.any() else None,
                          "ticks": int(stats[0]), "mean_batch": (stats[1] / stats[0]) if stats[0] else 0.0,
                          "peak_admitted_gb": stats[3] / 1e9, "busy_propagate_s": stats[4],
                          "busy_sac_s": stats[5], "busy_solvers_s": stats[6], "mac_timeouts": int(stats[7])}
                    for t, name in ((0, "propagate"), (1, "sac"), (2, "mac")):
                        sel = ok & (types == t)
                        if sel.any():
                            pt[name + "_p50_ms"] = float(np.percentile(lat[sel], 50))
                            pt[name + "_p99_ms"] = float(np.percentile(lat[sel], 99))
                    pts.append(pt)
                launches += srv.eA.launches + srv.eB.launches - l0
                results[mode] = {"points": pts, "register_s": reg_s}
    best = max(p["throughput_rps"] for p in results["batched"]["points"])
    best_plain = max(p["throughput_rps"] for p in results["plain"]["points"])
    line = {"metric": "served requests/s (propagate/SAC/MAC mix, p50/p99 latency)", "value": best,
            "unit": "requests/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64", "data": "synthetic (seeded generator)",
            "config": {"workload": SERVING_WORKLOAD.format(r=R), "networks": R, "slots_per_network": args.slots,
                       "max_batch": args.max_batch, "solvers": args.solvers,
                       "solve_time_limit_ms": args.solve_limit_ms, "rates_rps": rates,
                       "requests_per_rate": "min(%d, rate x %.1f s)" % (args.requests, args.duration),
                       "generate_s": gen_s},
            "batched": results["batched"], "plain": results["plain"],
            "batched_over_plain_peak_throughput": best / best_plain if best_plain else None,
            "gpu_launches": int(launches), "clocks": clk.summary(),
            "note": "latency = submit to result on the host (trace replayed by the native server); "
                    "throughput = requests / (last completion - first arrival) per rate point"}
    print(json.dumps(line))
    return 0


def run_gac(args):
    """Config-2 measurement: one GAC fixpoint of the large mixed network
    (binary rows + ternary positive tables, 20% of values removed) on the
    grid-wide persistent kernel; revisions/s and algorithmic GB/s. The
    published shape (500 tuples per table) has an empty GAC closure, so a
    second shape with 1200 tuples per table gives a full fixpoint."""
    import torch
    import cpim_gb300 as cp
    from oracle import pyoracle as O

    torch.cuda.set_device(0)
    peak, peak_kind = measured_peaks()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    eng = cp.Engine(0)
    out = []
    for ntup in (500, 1200):
        inst = cp.gen_mixed(2000, 64, 30000, 0.2, 0.5, 5000, ntup, 0.2, 1)
        net = eng.upload(inst, max_levels=2)
        sts = []
        for i in range(args.warmup + args.steps):
            net.dom_set(0, inst.init)
            flush.fill_(1)
            torch.cuda.synchronize()
            st = net.enforce_ac(0)
            if i >= args.warmup:
                sts.append(st)
        ms = statistics.median(s.device_ms for s in sts)
        st = sts[-1]
        t0 = time.perf_counter()
        ok, _, dels = O.gac(O.Instance(n=inst.n, W=inst.W, dom=inst.dom, init=inst.init,
                                       bx=inst.bin_scope[0::2].copy(), by=inst.bin_scope[1::2].copy(),
                                       brows=inst.bin_rows, tarity=inst.tab_arity, tscope=inst.tab_scope,
                                       tntup=inst.tab_ntup, ttup=inst.tab_tuples))
        cpu_s = time.perf_counter() - t0
        assert ok == (not st.inconsistent)
        if ok:
            assert dels == st.deletions
        ach = st.alg_bytes / (ms / 1e3) / 1e9
        out.append({"tuples_per_table": ntup, "inconsistent": bool(st.inconsistent), "ms": ms,
                    "revisions": int(st.revisions), "revisions_per_s": st.revisions / (ms / 1e3),
                    "deletions": int(st.deletions), "rounds": int(st.rounds),
                    "alg_gb_per_s": ach, "frac_of_hbm_peak": ach / peak,
                    "cpu_oracle_ms": cpu_s * 1e3, "cpu_oracle_cores": 1})
        net.close()
    # The level AC of the SAC sweep network (n=500, d=128, e=10000, p=0.40,
    # seed 7): every arc revised once, nothing removed.
    inst = cp.gen_binary(N, D, E, P, P, 0.0, SEED)
    net = eng.upload(inst, max_levels=2)
    sts = []
    for i in range(args.warmup + args.steps):
        net.dom_set(0, inst.init)
        flush.fill_(1)
        torch.cuda.synchronize()
        st = net.enforce_ac(0)
        if i >= args.warmup:
            sts.append(st)
    assert not sts[-1].inconsistent and sts[-1].deletions == 0
    ms = statistics.median(s.device_ms for s in sts)
    level_ac = {"workload": "AC fixpoint of the SAC sweep network (n=500 d=128 e=10000 p=0.40 seed 7), "
                            "L2 flushed before each run", "ms": ms, "revisions": int(sts[-1].revisions),
                "rounds": int(sts[-1].rounds), "alg_gb_per_s": sts[-1].alg_bytes / (ms / 1e3) / 1e9}
    net.close()
    eng.close()
    line = {"metric": "GAC revisions/s (single large mixed network, bit-exact)", "value": out[0]["revisions_per_s"],
            "unit": "revisions/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": out[0]["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64", "data": "synthetic (seeded generator)",
            "config": {"workload": "GAC fixpoint: n=2000 d=64, 30000 binary (p~U[0.2,0.5]) + 5000 ternary positive "
                                   "tables, 20% of values removed, seed 1; L2 flushed before each step",
                       "peak_source": peak_kind},
            "shapes": out, "sac_network_level_ac": level_ac}
    print(json.dumps(line))
    return 0


def run_tensor(args):
    """The tensor-core support-count tiles against the bitwise test on the
    benchmark network (see tensor_variant); `steps` timed repetitions."""
    import torch
    import cpim_gb300 as cp
    torch.cuda.set_device(0)
    inst = cp.gen_binary(N, D, E, P, P, 0.0, SEED)
    with cp.Engine(0) as eng:
        net = eng.upload(inst, max_levels=2)
        sweep_ms = None
        for _ in range(max(1, args.warmup)):
            st = net.enforce_sac1(0)
            sweep_ms = st.kernel_ms / max(1, st.sweeps)
        net.dom_set(0, inst.init)
        res = tensor_variant(inst, net, sweep_ms, reps=max(1, args.steps))
        net.close()
    line = {"metric": "SAC support-count tiles/s, tensor cores vs bitwise (bit-exact)",
            "value": res["tensor_cores"]["tiles_per_s"], "unit": "tiles/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 (0/1 operands, fp32 counts)", "data": "synthetic (seeded generator)",
            "config": bench_config(), **res}
    print(json.dumps(line))
    return 0


def run_xcsp(args):
    """The reference's own XCSP benchmark instances (a copy of its
    samples/bench directory given by --samples): MAC with dom/min and min
    value order to the first solution on the GPU (one device-resident search
    per instance, and all solved instances as one batched launch), checked
    against the reference's node counts (tests/golden/xcsp_reference_cases.json),
    beside the oracle's MAC on one host core and the reference's own solve
    time from that file (measured where the reference builds)."""
    import numpy as np
    import cpim_gb300 as cp
    from cpim_gb300.xcsp import read_xcsp
    from oracle import pyoracle as O
    with open(os.path.join(ROOT, "tests", "golden", "xcsp_reference_cases.json")) as f:
        cases = json.load(f)["cases"]
    rows = []
    with cp.Engine(0) as eng:
        solved_nets = []
        for c in cases:
            m = read_xcsp(os.path.join(args.samples, c["file"]))
            ref = c["mac"]
            if ref["time_out"]:
                rows.append({"file": c["file"], "reference": "time out at %d ms" % ref["solve_ms"]})
                continue
            reps = 3 if ref["num_positive"] < 5000 else 1
            best = 1e30
            for _ in range(reps):
                net = eng.upload(m.inst)  # a search leaves its levels changed
                t0 = time.perf_counter()
                r = net.mac_solve(time_limit_ms=300000)
                best = min(best, time.perf_counter() - t0)
                net.close()
            assert (r["num_positive"], r["num_negative"]) == (ref["num_positive"], ref["num_negative"]), c["file"]
            solved_nets.append((eng.upload(m.inst), m))
            row = {"file": c["file"], "n": m.inst.n, "constraints": m.inst.n_bin,
                   "nodes": ref["num_positive"] + ref["num_negative"], "solution": r["status"] == 1,
                   "gpu_ms": best * 1e3, "reference_cpu_ms": ref["solve_ms"]}
            if ref["num_positive"] < 50000:
                from tests.golden_cases import oracle_view_of
                t0 = time.perf_counter()
                O.mac(oracle_view_of(m.inst))
                row["oracle_cpu_ms"] = (time.perf_counter() - t0) * 1e3
            rows.append(row)
        t0 = time.perf_counter()
        mb = cp.MacBatch(eng, [(n, []) for n, _ in solved_nets], time_limit_ms=300000)
        res = mb.wait()
        batch_s = time.perf_counter() - t0
        mb.close()
        for n, _ in solved_nets:
            n.close()
    nodes = sum(r["num_positive"] + r["num_negative"] for r in res)
    line = {"metric": "MAC first-solution searches on the reference's XCSP instances (node counts bit-exact)",
            "value": len(res) / batch_s, "unit": "solves/s", "n_gpus": 1, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "the reference's samples/bench XCSP files",
            "config": {"workload": "MAC(AC_3bit, dom/min, min value) on samples/bench (queens, composed-25-1-2, "
                                   "rand-2-23; haystacks-11 exceeds the reference's 60 s limit)"},
            "batch": {"searches": len(res), "wall_s": batch_s, "nodes_per_s": nodes / batch_s},
            "instances": rows}
    print(json.dumps(line))
    return 0


def run_mac(args):
    """Config-1 measurement: MAC (dom/min, min value) to the first solution on
    the plain CPU-runnable shape, seeds 1..10: the device search (one CTA per
    search), the host-driven search (one launch per node), a batch of all
    searches in one launch, and the oracle's CPU MAC."""
    import cpim_gb300 as cp
    from oracle import pyoracle as O

    insts = [cp.gen_binary(50, 16, 250, 0.30, 0.30, 0.0, s) for s in range(1, 11)]
    res = {}
    nodes = None
    for mode, name in ((0, "device_search"), (1, "host_driven")):
        with cp.Engine(0) as eng:
            eng.set_search_mode(mode)
            nets = [eng.upload(i) for i in insts]
            for n in nets[:2]:
                n.mac_solve()
            t0 = time.perf_counter()
            rs = [n.mac_solve() for n in nets]
            wall = time.perf_counter() - t0
            nn = sum(r["num_positive"] + r["num_negative"] for r in rs)
            nodes = nn if nodes is None else nodes
            assert nn == nodes
            res[name] = {"ms_per_solve": wall * 1e3 / len(nets), "nodes_per_s": nn / wall}
            for n in nets:
                n.close()
    with cp.Engine(0) as eng:
        nets = [eng.upload(i) for i in insts]
        reps = 64
        jobs = [(n, []) for n in nets] * reps
        mb = cp.MacBatch(eng, jobs[:10])
        mb.wait()
        mb.close()
        t0 = time.perf_counter()
        mb = cp.MacBatch(eng, jobs)
        rs = mb.wait()
        wall = time.perf_counter() - t0
        mb.close()
        nn = sum(r["num_positive"] + r["num_negative"] for r in rs)
        res["device_batch"] = {"searches": len(jobs), "ms_total": wall * 1e3, "solves_per_s": len(jobs) / wall,
                               "nodes_per_s": nn / wall}
        for n in nets:
            n.close()
    t0 = time.perf_counter()
    for i in insts:
        O.mac(O.Instance(n=i.n, W=i.W, dom=i.dom, init=i.init, bx=i.bin_scope[0::2].copy(),
                         by=i.bin_scope[1::2].copy(), brows=i.bin_rows, tarity=i.tab_arity, tscope=i.tab_scope,
                         tntup=i.tab_ntup, ttup=i.tab_tuples))
    cpu = time.perf_counter() - t0
    res["cpu_oracle_1core"] = {"ms_per_solve": cpu * 1e3 / len(insts), "nodes_per_s": nodes / cpu}
    line = {"metric": "MAC first-solution solves/s (cfg1, node counts bit-exact)",
            "value": res["device_batch"]["solves_per_s"], "unit": "solves/s", "n_gpus": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (seeded generator)",
            "config": {"workload": "MAC(AC_3bit, dom/min, min): n=50 d=16 e=250 p=0.30, seeds 1..10",
                       "nodes_total_10_seeds": nodes},
            "modes": res}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 20 for the SAC sweep, whose step is 128 closures; 3 for the "
                         "uneven batch, whose step is a full AC + SAC1 of 4096 instances; 300 otherwise)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="timed steps only (for profiling)")
    ap.add_argument("--closures-per-step", type=int, default=128,
                    help="SAC closures per timed step of the default workload")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload without the GAC and uneven-batch samples")
    ap.add_argument("--workload", default="sac", choices=["sac", "uneven", "serving", "gac", "mac", "tensor", "xcsp"],
                    help="sac: the batched SAC sweep (headline); uneven: the uneven multi-instance batch; "
                         "serving: the request server under Poisson load; gac: the large GAC fixpoint; "
                         "mac: MAC searches on the plain shape; tensor: support-count tiles on the tensor cores "
                         "against the bitwise test; xcsp: MAC on the reference's XCSP instances (--samples)")
    ap.add_argument("--instances", type=int, default=4096, help="uneven workload: instances")
    ap.add_argument("--samples", default="", help="xcsp workload: a copy of the reference's samples/bench directory")
    ap.add_argument("--per-instance-sample", type=int, default=256, help="uneven workload: one-by-one sample")
    ap.add_argument("--networks", type=int, default=64, help="serving: resident networks")
    ap.add_argument("--slots", type=int, default=16, help="serving: working levels per resident network")
    ap.add_argument("--rates", default="100,300,1000,3000,10000,50000", help="serving: offered loads, req/s")
    ap.add_argument("--requests", type=int, default=2000, help="serving: most requests per rate point")
    ap.add_argument("--duration", type=float, default=2.0, help="serving: seconds of arrivals per rate point")
    ap.add_argument("--max-batch", type=int, default=256, help="serving: requests per batch tick")
    ap.add_argument("--solvers", type=int, default=4, help="serving: MAC solver threads")
    ap.add_argument("--solve-limit-ms", type=int, default=500, help="serving: MAC solve time limit")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 3 if args.workload == "uneven" and args.impl == "ours" else (20 if args.workload == "sac" else 300)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "uneven":
        return run_uneven(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "gac":
        return run_gac(args)
    if args.workload == "mac":
        return run_mac(args)
    if args.workload == "tensor":
        return run_tensor(args)
    if args.workload == "xcsp":
        return run_xcsp(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
