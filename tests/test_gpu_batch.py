"""GPU tests of multi-instance batches: one launch per phase for all members,
the sweep replayed from a CUDA graph; every member's result must equal its
own single-instance result and the oracle's."""
import numpy as np
import pytest

import cpim_gb300 as cp
from oracle import pyoracle as O
from tests.golden_cases import oracle_view_of

pytestmark = pytest.mark.gpu


def _members(count=24, seed=5):
    insts = [cp.gen_uneven(seed * 1000003 + i, 20, 60, 256) for i in range(count)]
    # Tight members: SAC removes values, some are inconsistent.
    insts += [cp.gen_binary(30, 8, 120, 0.35, 0.35, 0.1, s) for s in (1, 2, 4)]
    insts += [cp.gen_binary(30, 8, 120, 0.45, 0.45, 0.1, s) for s in (1, 2)]
    insts += [cp.gen_binary(40, 100, 160, 0.8, 0.8, 0.2, 3)]
    return insts


def _single(inst):
    with cp.Engine(0) as eng:
        net = eng.upload(inst, max_levels=2)
        st = net.enforce_sac1(0)
        d = net.dom_get(0)
        net.close()
    return bool(st.inconsistent), d, st.deletions


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_sac_matches_single_and_oracle(graphs):
    insts = _members()
    with cp.Engine(0) as eng:
        nets = [eng.upload(i, max_levels=2) for i in insts]
        b = cp.Batch(eng, nets)
        b.set_graphs(graphs)
        st, inc = b.sac1()
        assert st.branches > 0
        for k, (inst, net) in enumerate(zip(insts, nets)):
            s_inc, s_dom, _ = _single(inst)
            assert bool(inc[k]) == s_inc, k
            if not s_inc:
                assert np.array_equal(net.dom_get(0), s_dom), k
            if k % 4 == 0:
                ok, d, _ = O.sac1(oracle_view_of(inst))
                assert ok == (not inc[k]), k
                if ok:
                    assert np.array_equal(net.dom_get(0), d), k
        b.close()
        for n in nets:
            n.close()


def test_batch_ac_matches_oracle():
    insts = _members(16, 9)
    with cp.Engine(0) as eng:
        nets = [eng.upload(i, max_levels=2) for i in insts]
        b = cp.Batch(eng, nets)
        st, inc = b.ac()
        for k, (inst, net) in enumerate(zip(insts, nets)):
            ok, d, _ = O.ac3bit(oracle_view_of(inst))
            assert ok == (not inc[k]), k
            if ok:
                assert np.array_equal(net.dom_get(0), d), k
        b.close()


def test_batch_groups_and_tuning(tmp_path, monkeypatch):
    monkeypatch.setenv("CPGPU_TUNE_CACHE", str(tmp_path / "tune.txt"))
    insts = _members(12, 3)
    with cp.Engine(0) as eng:
        nets = [eng.upload(i, max_levels=2) for i in insts]
        b = cp.Batch(eng, nets)
        info = b.info(0)
        assert info["groups"] >= 2  # several domain widths
        b.tune()
        assert (tmp_path / "tune.txt").exists()
        st, inc = b.sac1()
        for k, inst in enumerate(insts):
            s_inc, s_dom, _ = _single(inst)
            assert bool(inc[k]) == s_inc
            if not s_inc:
                assert np.array_equal(nets[k].dom_get(0), s_dom)
        # A second batch over the same shapes reads the cached choice.
        b2 = cp.Batch(eng, nets)
        assert b2.info(0)["tiled"] == b.info(0)["tiled"]
        b.close()
        b2.close()


def test_batch_with_tables_matches_oracle():
    insts = [cp.gen_mixed(40, 8, 100, 0.2, 0.3, 15, 350, 0.0, s) for s in (1, 2)]
    insts += [cp.gen_mixed(30, 8, 60, 0.25, 0.45, 20, 120, 0.1, s) for s in (1, 2)]
    with cp.Engine(0) as eng:
        nets = [eng.upload(i, max_levels=2) for i in insts]
        b = cp.Batch(eng, nets)
        st, inc = b.sac1()
        for k, inst in enumerate(insts):
            ok, d, _ = O.sac1(oracle_view_of(inst))
            assert ok == (not inc[k])
            if ok:
                assert np.array_equal(nets[k].dom_get(0), d)
        b.close()


def test_device_generator_matches_host():
    with cp.Engine(0) as eng:
        for args in [(50, 16, 250, 0.3, 0.3, 0.0, 1), (40, 100, 160, 0.8, 0.8, 0.2, 3), (60, 256, 300, 0.5, 0.5, 0.1, 2)]:
            inst = cp.gen_binary(*args)
            net = cp.upload_binary_device(eng, *args, max_levels=2)
            assert np.array_equal(net.rows(inst.bin_rows.size), inst.bin_rows)
            assert np.array_equal(net.dom_get(0), inst.init)
            net.close()
        for s in range(6):
            seed = 7 * 1000003 + s
            inst = cp.gen_uneven(seed, 20, 120, 256)
            net = cp.upload_uneven_device(eng, seed, 20, 120, 256, max_levels=2)
            assert (net.n, net.W) == (inst.n, inst.W)
            assert np.array_equal(net.rows(inst.bin_rows.size), inst.bin_rows)
            st = net.enforce_sac1(0)
            ref = eng.upload(inst, max_levels=2)
            st2 = ref.enforce_sac1(0)
            assert st.inconsistent == st2.inconsistent
            if not st.inconsistent:
                assert np.array_equal(net.dom_get(0), ref.dom_get(0))
            net.close()
            ref.close()


def test_batch_copy_level_restores():
    insts = _members(8, 11)
    with cp.Engine(0) as eng:
        nets = [eng.upload(i, max_levels=2) for i in insts]
        for n in nets:
            n.level_copy(0, 1)
        b = cp.Batch(eng, nets)
        st1, inc1 = b.sac1()
        d1 = [n.dom_get(0) for n in nets]
        b.copy_level(1)
        for n, inst in zip(nets, insts):
            assert np.array_equal(n.dom_get(0), inst.init)
        st2, inc2 = b.sac1()
        assert np.array_equal(inc1, inc2)
        for n, d, bad in zip(nets, d1, inc1):
            if not bad:  # after a wipe-out only the verdict is defined
                assert np.array_equal(n.dom_get(0), d)
        b.close()


def _edits_for(inst, rng, count):
    """Random (var, val) choices with val in the variable's initial domain."""
    out = []
    for _ in range(count):
        x = int(rng.integers(0, inst.n))
        words = inst.init[x * inst.W:(x + 1) * inst.W]
        vals = [w * 64 + b for w in range(inst.W) for b in range(64) if (int(words[w]) >> b) & 1]
        out.append((x, int(vals[int(rng.integers(0, len(vals)))])))
    return out


@pytest.mark.parametrize("op", ["ac", "sac1"])
def test_batch_levels_one_network_many_queries(op):
    """One resident network queried on several levels in one batch, with
    per-query variable choices, beside other networks: each member equals the
    same query run alone; the gathered domains equal per-member reads."""
    rng = np.random.default_rng(17)
    shared = cp.gen_uneven(424242, 40, 80, 64)
    others = [cp.gen_uneven(31337 + i, 20, 60, 128) for i in range(3)]
    slots = 5
    with cp.Engine(0) as eng:
        net_s = eng.upload(shared, max_levels=1 + slots)
        net_o = [eng.upload(i, max_levels=2) for i in others]
        members = [net_s] * slots + net_o
        levels = list(range(1, slots + 1)) + [1] * len(net_o)
        b = cp.Batch(eng, members, levels=levels)
        queries = [_edits_for(shared, rng, k % 3) for k in range(slots)] + [_edits_for(o, rng, 1) for o in others]
        edits = [(m, x, a) for m, q in enumerate(queries) for x, a in q]
        b.load(0, edits)
        st, inc = (b.ac() if op == "ac" else b.sac1())
        doms = b.dom_get()
        insts = [shared] * slots + others
        for m, (inst, q) in enumerate(zip(insts, queries)):
            with cp.Engine(0) as e1:
                one = e1.upload(inst, max_levels=2)
                for x, a in q:
                    one.reduce_to(0, x, a)
                s1 = one.enforce_ac(0) if op == "ac" else one.enforce_sac1(0)
                assert bool(inc[m]) == bool(s1.inconsistent), m
                if not s1.inconsistent:
                    assert np.array_equal(doms[m], one.dom_get(0)), m
                one.close()
        # Level 0 of the shared network is untouched by the queries.
        assert np.array_equal(net_s.dom_get(0), shared.init)
        b.close()
        net_s.close()
        for n in net_o:
            n.close()


def test_batch_rejects_repeated_member_level():
    inst = cp.gen_uneven(5, 20, 30, 16)
    with cp.Engine(0) as eng:
        net = eng.upload(inst, max_levels=3)
        with pytest.raises(cp.CPError):
            cp.Batch(eng, [net, net], levels=[1, 1])
        b = cp.Batch(eng, [net, net], levels=[1, 2])
        with pytest.raises(cp.CPError):
            b.load(0, [(0, inst.n, 0)])  # variable out of range
        with pytest.raises(cp.CPError):
            b.load(0, [(2, 0, 0)])  # member out of range
        b.close()
        net.close()


@pytest.mark.parametrize("quota", [1, 3])
def test_batch_cta_quota_and_priority_keep_results(quota):
    """Retiring sweep CTAs (quota) on a low-priority stream, with members
    uploaded on another engine, give the persistent sweep's results."""
    insts = _members(10, 21)
    with cp.Engine(0) as up, cp.Engine(0) as eq, cp.Engine(0) as ep:
        eq.set_priority(-1)
        eq.set_cta_quota(quota)
        ep.set_priority(1)
        nets = [up.upload(i, max_levels=3) for i in insts]
        for n in nets:
            n.level_copy(0, 1)
            n.level_copy(0, 2)
        bq = cp.Batch(eq, nets, level=1)
        bp = cp.Batch(ep, nets, level=2)
        sq, iq = bq.sac1()
        sp, ip = bp.sac1()
        assert np.array_equal(iq, ip)
        dq, dp = bq.dom_get(), bp.dom_get()
        for k in range(len(nets)):
            if not ip[k]:
                assert np.array_equal(dq[k], dp[k]), k
        # Branch and deletion totals are not compared: failed branches remove
        # their value at once, so how many branches a sweep still tests, and
        # how many values an inconsistent member loses before its wipe-out is
        # seen, depend on timing. The closures above are what must agree.
        bq.close()
        bp.close()
        for n in nets:
            n.close()
