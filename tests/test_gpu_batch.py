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
