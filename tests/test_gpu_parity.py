"""GPU parity: the engine's results through the C ABI against the reference's
own outputs (golden fixtures) and the CPU oracle. Bit-exact: final domain
words, verdicts, deletion counts, MAC node counts and first solutions."""
import numpy as np
import pytest

import cpim_gb300 as cp
from oracle import pyoracle as O
from tests.golden_cases import dom_hex, make_engine_instance, oracle_view_of

pytestmark = pytest.mark.gpu


def _cases(golden, op, names=None):
    return [c for c in golden if c["op"] == op and (names is None or c["name"] in names)]


def test_ac_matches_reference(engine, golden):
    cases = _cases(golden, "ac3bit")
    assert cases
    for c in cases:
        inst = make_engine_instance(c["args"])
        net = engine.upload(inst)
        st = net.enforce_ac(0)
        r = c["result"]
        assert bool(st.inconsistent) == (not r["consistent"]), c["args"]
        if r["consistent"]:
            assert st.deletions == r["deletions"], c["args"]
            assert dom_hex(net.dom_get(0)) == r["domains"], c["args"]
        net.close()


def test_sac1_matches_reference(engine, golden):
    cases = _cases(golden, "sac1")
    assert cases
    for c in cases:
        inst = make_engine_instance(c["args"])
        net = engine.upload(inst)
        st = net.enforce_sac1(0)
        r = c["result"]
        assert bool(st.inconsistent) == (not r["consistent"]), c["args"]
        if r["consistent"]:
            assert st.deletions == r["deletions"], c["args"]
            assert dom_hex(net.dom_get(0)) == r["domains"], c["args"]
        net.close()


@pytest.mark.parametrize("mode", [0, 1], ids=["device-search", "host-driven"])
def test_mac_matches_reference(golden, mode):
    cases = _cases(golden, "mac")
    assert cases
    with cp.Engine(0) as engine:
        engine.set_search_mode(mode)
        for c in cases:
            inst = make_engine_instance(c["args"])
            net = engine.upload(inst)
            m = net.mac_solve(time_limit_ms=60000)
            r = c["result"]
            assert m["num_positive"] == r["num_positive"], c["args"]
            assert m["num_negative"] == r["num_negative"], c["args"]
            assert (m["status"] == 1) == (r["num_sol"] == 1), c["args"]
            if m["status"] == 1:
                assert m["solution"] == r["solution"], c["args"]
            net.close()


@pytest.mark.parametrize("args", [(60, 8, 150, 0.2, 0.4, 20, 300, 0.1), (60, 16, 200, 0.2, 0.4, 30, 2000, 0.1),
                                  (40, 8, 100, 0.3, 0.5, 30, 150, 0.1), (30, 8, 60, 0.3, 0.5, 40, 60, 0.2)])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_gac_mixed_matches_oracle(engine, args, seed):
    inst = cp.gen_mixed(*args, seed)
    ok, d, dels = O.gac(oracle_view_of(inst))
    net = engine.upload(inst)
    st = net.enforce_ac(0)
    assert bool(st.inconsistent) == (not ok)
    if ok:
        assert st.deletions == dels
        assert np.array_equal(net.dom_get(0), d)
    net.close()


@pytest.mark.parametrize("args", [(40, 8, 100, 0.2, 0.3, 15, 350, 0.0), (30, 8, 60, 0.25, 0.45, 20, 120, 0.1)])
def test_sac_mixed_matches_oracle(engine, args):
    for seed in (1, 2):
        inst = cp.gen_mixed(*args, seed)
        ok, d, dels = O.sac1(oracle_view_of(inst))
        net = engine.upload(inst)
        st = net.enforce_sac1(0)
        assert bool(st.inconsistent) == (not ok)
        if ok:
            assert np.array_equal(net.dom_get(0), d)
            assert st.deletions == dels
        net.close()


@pytest.mark.parametrize("args", [(30, 8, 120, 0.35, 0.35, 0.1, 1), (30, 8, 120, 0.35, 0.35, 0.1, 4),
                                  (30, 8, 120, 0.45, 0.45, 0.1, 3), (40, 100, 160, 0.8, 0.8, 0.2, 3),
                                  (24, 256, 60, 0.9, 0.9, 0.3, 3), (60, 64, 600, 0.55, 0.55, 0.1, 5),
                                  (100, 128, 1000, 0.4, 0.4, 0.0, 7), (150, 16, 3000, 0.3, 0.3, 0.05, 2),
                                  (60, 300, 500, 0.5, 0.5, 0.0, 4), (120, 64, 2000, 0.5, 0.5, 0.0, 8),
                                  (80, 128, 1500, 0.55, 0.55, 0.0, 6), (40, 70, 200, 0.88, 0.88, 0.0, 4)])
def test_sac_tiled_equals_general(args):
    # The tiled sweep (two-round test, deeper branches handed to the general
    # kernel) and the general per-branch kernel give the same SAC closure,
    # which is the oracle's.
    inst = cp.gen_binary(*args)
    ok_o, d_o, dels_o = O.sac1(oracle_view_of(inst))
    out = []
    for mode in (0, 1):
        with cp.Engine(0) as eng:
            eng.set_sac_mode(mode)
            net = eng.upload(inst)
            st = net.enforce_sac1(0)
            out.append((bool(st.inconsistent), net.dom_get(0), st.deletions, st.branches))
            net.close()
    for inc, d, dels, _ in out:
        assert inc == (not ok_o)
        if ok_o:
            assert np.array_equal(d, d_o)
            assert dels == dels_o


def test_singletons_batched_plain_oracle(engine):
    inst = cp.gen_binary(100, 128, 1000, 0.4, 0.4, 0.0, 7)
    ov = oracle_view_of(inst)
    net = engine.upload(inst)
    rng = np.random.default_rng(5)
    xs = rng.integers(0, inst.n, 300).astype(np.int32)
    avals = rng.integers(0, 128, 300).astype(np.int32)
    ok_b, st_b = net.singletons(xs, avals, mode=0)
    ok_p, st_p = net.singletons(xs, avals, mode=1)
    assert np.array_equal(ok_b, ok_p)
    d0 = inst.init.copy()
    for i in range(0, 300, 10):
        assert bool(ok_b[i]) == O.singleton(ov, d0, int(xs[i]), int(avals[i]))
    assert st_b.branches == 300 and st_p.launches == 300
    net.close()


def test_singletons_tight_failures(engine):
    # Tight network where many singleton tests fail: batched == plain == oracle.
    # Singleton tests run on an AC-closed level, as in SAC1 (the closure of
    # the level with x reduced to a is then unique).
    for seed in (2, 3):
        inst = cp.gen_binary(30, 8, 120, 0.45, 0.45, 0.1, seed)
        ov = oracle_view_of(inst)
        net = engine.upload(inst)
        st = net.enforce_ac(0)
        assert not st.inconsistent
        dom = net.dom_get(0)
        okc, d_or, _ = O.ac3bit(ov)
        assert okc and np.array_equal(dom, d_or)
        xs, vs = [], []
        for x in range(inst.n):
            for a in range(8):
                if (int(dom[x]) >> a) & 1:
                    xs.append(x)
                    vs.append(a)
        ok_b, _ = net.singletons(xs, vs, mode=0)
        ok_p, _ = net.singletons(xs, vs, mode=1)
        assert np.array_equal(ok_b, ok_p)
        ref = [O.singleton(ov, dom, x, a) for x, a in zip(xs, vs)]
        assert ok_b.astype(bool).tolist() == ref
        assert 0 < sum(ref) < len(ref)
        net.close()


@pytest.mark.parametrize("args", [(800, 64, 6000, 0.2, 0.5, 1500, 1000, 0.2, 11),
                                  (800, 64, 6000, 0.2, 0.5, 1500, 500, 0.2, 11),
                                  (2000, 64, 30000, 0.2, 0.5, 5000, 1200, 0.2, 1),
                                  (2000, 64, 30000, 0.2, 0.5, 5000, 500, 0.2, 1)])
def test_grid_kernel_large_mixed_matches_oracle(engine, args):
    # More than 8192 arc+table incidences: the single-instance fixpoint runs on
    # the whole grid (cooperative persistent kernel). The last case is the
    # full mixed-arity workload (n=2000, d=64, 30000 binary + 5000 ternary
    # tables of 500 tuples, 20% of values removed), whose GAC closure is empty.
    inst = cp.gen_mixed(*args)
    ok, d, dels = O.gac(oracle_view_of(inst))
    net = engine.upload(inst)
    st = net.enforce_ac(0)
    assert bool(st.inconsistent) == (not ok)
    if ok:
        assert st.deletions == dels
        assert np.array_equal(net.dom_get(0), d)
        # Idempotent: a second pass removes nothing.
        st2 = net.enforce_ac(0)
        assert st2.deletions == 0 and not st2.inconsistent
    net.close()


def test_grid_kernel_binary_matches_oracle(engine):
    inst = cp.gen_binary(2000, 64, 30000, 0.2, 0.5, 0.2, 3)
    ok, d, dels = O.ac3bit(oracle_view_of(inst))
    net = engine.upload(inst)
    st = net.enforce_ac(0)
    assert bool(st.inconsistent) == (not ok)
    if ok:
        assert st.deletions == dels
        assert np.array_equal(net.dom_get(0), d)
    net.close()


def test_gsolver_solution_valid(engine):
    for seed in range(1, 6):
        inst = cp.gen_binary(50, 16, 250, 0.3, 0.3, 0.0, seed)
        net = engine.upload(inst)
        g = net.gsolver_solve(time_limit_ms=60000)
        m = O.mac(oracle_view_of(inst))
        assert (g["status"] == 1) == (m["status"] == 1)
        if g["status"] == 1:
            assert O.check_solution(oracle_view_of(inst), g["solution"])
        net.close()


def test_level_ops_round_trip(engine):
    inst = cp.gen_binary(20, 100, 40, 0.5, 0.5, 0.0, 4)
    net = engine.upload(inst, max_levels=4)
    d0 = net.dom_get(0)
    assert np.array_equal(d0, inst.init)
    net.level_copy(0, 1)
    net.reduce_to(1, 3, 77)
    d1 = net.dom_get(1)
    assert net.sizes(1)[3] == 1 and (int(d1[3 * 2 + 1]) >> (77 - 64)) & 1
    net.remove(1, 4, 5)
    assert net.sizes(1)[4] == 99
    assert np.array_equal(net.dom_get(0), d0)
    with pytest.raises(cp.CPError):
        net.reduce_to(1, 3, 100)
    with pytest.raises(cp.CPError):
        net.level_copy(0, 4)
    net.dom_set(2, d0)
    assert np.array_equal(net.dom_get(2), d0)
    net.close()


@pytest.mark.parametrize("p", [0.5, 0.6])
def test_sac_tiled_with_repeated_pairs(p):
    # Two constraints on the same variable pair (the union of two networks
    # over the same variables): the tiled sweep ANDs both rows into one
    # neighbour slot, and must still give the oracle's SAC closure (0.5:
    # consistent, 0.6: SAC wipe-out).
    a = cp.gen_binary(30, 64, 200, p, p, 0.0, 11)
    b = cp.gen_binary(30, 64, 200, p, p, 0.0, 12)
    pairs_a = {tuple(sorted(p)) for p in a.bin_scope.reshape(-1, 2).tolist()}
    pairs_b = {tuple(sorted(p)) for p in b.bin_scope.reshape(-1, 2).tolist()}
    assert pairs_a & pairs_b  # the union repeats some pairs
    inst = cp.Instance(n=a.n, W=a.W, dom=a.dom, init=a.init,
                       bin_scope=np.concatenate([a.bin_scope, b.bin_scope]),
                       bin_rows=np.concatenate([a.bin_rows, b.bin_rows]),
                       tab_arity=a.tab_arity, tab_scope=a.tab_scope, tab_ntup=a.tab_ntup,
                       tab_tuples=a.tab_tuples)
    ok_o, d_o, dels_o = O.sac1(oracle_view_of(inst))
    for mode in (0, 1):
        with cp.Engine(0) as eng:
            eng.set_sac_mode(mode)
            net = eng.upload(inst)
            st = net.enforce_sac1(0)
            assert bool(st.inconsistent) == (not ok_o), mode
            if ok_o:
                assert np.array_equal(net.dom_get(0), d_o), mode
                assert st.deletions == dels_o, mode
            net.close()


@pytest.mark.parametrize("args", [(500, 12, 4500, 0.5, 0.5, 0.0, 1), (500, 12, 4500, 0.51, 0.51, 0.0, 1),
                                  (100, 128, 1000, 0.4, 0.4, 0.0, 7), (40, 70, 200, 0.88, 0.88, 0.0, 4)])
def test_sac_graph_rounds_equal_direct(args):
    # SAC1 rounds replayed as CUDA graphs (the root-AC round and the
    # events-AC round, captured per level) give the oracle's closure, as the
    # uncaptured launches do, across levels and repeated calls. The first two
    # networks take the grid AC path and need several sweeps (the second ends
    # in a wipe-out).
    inst = cp.gen_binary(*args)
    ok_o, d_o, dels_o = O.sac1(oracle_view_of(inst))
    for graphs in (True, False):
        with cp.Engine(0) as eng:
            eng.set_graphs(graphs)
            net = eng.upload(inst, max_levels=3)
            for _ in range(2):
                for level in (0, 1):
                    net.dom_set(level, inst.init)
                    st = net.enforce_sac1(level)
                    assert bool(st.inconsistent) == (not ok_o), (graphs, level)
                    if ok_o:
                        assert np.array_equal(net.dom_get(level), d_o), (graphs, level)
                        assert st.deletions == dels_o, (graphs, level)
            net.close()


def test_reload_sync_and_async_match_oracle():
    # cp_net_reload / cp_net_reload_async replace the relations and domains of
    # an uploaded network with those of another instance of the same shape;
    # two engines alternate with the next reload queued while the current
    # closure runs, and every closure equals the oracle's SAC1 of the
    # instance it was given.
    base = cp.gen_binary(60, 24, 300, 0.45, 0.45, 0.1, 3)
    rng = np.random.default_rng(11)
    insts = []
    for k in range(4):  # same scopes, other rows and initial domains
        keep = rng.integers(0, 2 ** 63, size=base.bin_rows.shape, dtype=np.int64).astype(np.uint64)
        keep |= rng.integers(0, 2 ** 63, size=base.bin_rows.shape, dtype=np.int64).astype(np.uint64)
        init = base.init & ~(np.uint64(1) << rng.integers(0, 24, size=base.init.shape).astype(np.uint64))
        insts.append(cp.Instance(n=base.n, W=base.W, dom=base.dom, init=init, bin_scope=base.bin_scope,
                                 bin_rows=base.bin_rows & keep, tab_arity=base.tab_arity, tab_scope=base.tab_scope,
                                 tab_ntup=base.tab_ntup, tab_tuples=base.tab_tuples))
    want = [O.sac1(oracle_view_of(i)) for i in insts]
    with cp.Engine(0) as e1, cp.Engine(0) as e2:
        nets = (e1.upload(base, max_levels=2), e2.upload(base, max_levels=2))
        for k, inst in enumerate(insts):
            nets[0].reload(inst)
            st = nets[0].enforce_sac1(0)
            ok, d, dels = want[k]
            assert bool(st.inconsistent) == (not ok)
            if ok:
                assert np.array_equal(nets[0].dom_get(0), d)
        order = [2, 0, 3, 1, 1, 2]
        nets[0].reload_async(insts[order[0]])
        for i, k in enumerate(order):
            cur = nets[i % 2]
            if i + 1 < len(order):
                nets[(i + 1) % 2].reload_async(insts[order[i + 1]])
            st = cur.enforce_sac1(0)
            ok, d, dels = want[k]
            assert bool(st.inconsistent) == (not ok), (i, k)
            if ok:
                assert np.array_equal(cur.dom_get(0), d), (i, k)
                assert st.deletions == dels
        # A host write of the domains right after an asynchronous reload waits
        # for the reload's copy out of the shared staging buffer.
        nets[0].reload_async(insts[0])
        nets[0].dom_set(0, insts[1].init)
        nets[0].reload(insts[1])
        st = nets[0].enforce_sac1(0)
        ok, d, _ = want[1]
        assert bool(st.inconsistent) == (not ok)
        if ok:
            assert np.array_equal(nets[0].dom_get(0), d)
        for n in nets:
            n.close()


def test_level_push_pop_and_set_var():
    # Network::NewLevel / BackTo over the C ABI (cp_level_push / cp_level_pop_to)
    # and the per-variable domain write (cp_dom_set_var).
    inst = cp.gen_binary(40, 20, 150, 0.35, 0.35, 0.1, 9)
    with cp.Engine(0) as eng:
        net = eng.upload(inst, max_levels=4)
        assert net.level_top() == 0
        d0 = net.dom_get(0)
        assert net.level_push(0) == 1 and net.level_top() == 1
        assert np.array_equal(net.dom_get(1), d0)
        net.reduce_to(1, 3, int(np.flatnonzero([(int(d0[3]) >> a) & 1 for a in range(20)])[0]))
        net.enforce_ac(1)
        assert np.array_equal(net.dom_get(0), d0)  # the pushed level leaves level 0 alone
        assert net.level_push(1) == 2 and net.level_push(2) == 3
        with pytest.raises(cp.CPError):
            net.level_push(3)  # no level 4
        net.level_pop_to(1)
        assert net.level_top() == 1
        # Per-variable write, bits past the domain size cleared.
        net.dom_set_var(2, 5, np.array([np.uint64(0xFFFFFFFFFFFFFFFF)], np.uint64))
        d2 = net.dom_get(2)
        assert int(d2[5]) == (1 << 20) - 1
        words = net.dom_get(1)
        words[5] = np.uint64(0b1011)
        net.dom_set_var(1, 5, words[5:6])
        assert np.array_equal(net.dom_get(1), words)
        ok, d, dels = O.ac3bit(oracle_view_of(cp.Instance(n=inst.n, W=inst.W, dom=inst.dom, init=words,
                                                          bin_scope=inst.bin_scope, bin_rows=inst.bin_rows,
                                                          tab_arity=inst.tab_arity, tab_scope=inst.tab_scope,
                                                          tab_ntup=inst.tab_ntup, tab_tuples=inst.tab_tuples)))
        st = net.enforce_ac(1)
        assert bool(st.inconsistent) == (not ok)
        if ok:
            assert np.array_equal(net.dom_get(1), d)
        with pytest.raises(cp.CPError):
            net.dom_set_var(1, inst.n, words[:1])
        net.close()


def test_sac1_begin_end_equals_enforce():
    # cp_enforce_sac1_begin / _end give the closure and stats of
    # cp_enforce_sac1 (including closures of several sweeps and wipe-outs),
    # and refuse a second begin or an end without a begin.
    cases = [(60, 16, 300, 0.35, 0.35, 0.1, 3), (30, 8, 120, 0.45, 0.45, 0.1, 3), (40, 100, 160, 0.8, 0.8, 0.2, 3)]
    with cp.Engine(0) as eng:
        for args in cases:
            inst = cp.gen_binary(*args)
            ok, d, dels = O.sac1(oracle_view_of(inst))
            net = eng.upload(inst, max_levels=2)
            net.enforce_sac1_begin(0)
            with pytest.raises(cp.CPError):
                net.enforce_sac1_begin(0)
            st = net.enforce_sac1_end()
            assert bool(st.inconsistent) == (not ok)
            if ok:
                assert st.deletions == dels
                assert np.array_equal(net.dom_get(0), d)
            with pytest.raises(cp.CPError):
                net.enforce_sac1_end()
            net.dom_set(0, inst.init)
            st2 = net.enforce_sac1(0)
            assert (st2.inconsistent, st2.deletions, st2.sweeps) == (st.inconsistent, st.deletions, st.sweeps)
            # _end_domains returns the closure with the call.
            net.dom_set(0, inst.init)
            net.enforce_sac1_begin(0)
            st3, d3 = net.enforce_sac1_end_domains()
            assert (st3.inconsistent, st3.deletions, st3.sweeps) == (st.inconsistent, st.deletions, st.sweeps)
            if ok:
                assert np.array_equal(d3, d)
                assert np.array_equal(net.dom_get(0), d)
            net.close()
