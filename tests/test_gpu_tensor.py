"""GPU test of the SAC support-count tiles (cp_sac_tiles): the tensor-core
product (tcgen05, bf16 0/1 operands, fp32 counts in tensor memory) and the
bitwise AND-then-any give the same removal words, and both equal a numpy
count of supports computed from the network's rows."""
import numpy as np
import pytest

import cpim_gb300 as cp

pytestmark = pytest.mark.gpu


def _bits(words, d):
    """Bool vector of the first d values of a W-word domain or row."""
    out = np.zeros(d, bool)
    for a in range(d):
        out[a] = (int(words[a >> 6]) >> (a & 63)) & 1
    return out


def _rows(inst, c, first):
    """Rows of constraint c: first=True, rows of bx over by; else by over bx."""
    W = inst.W
    bx, by = inst.bin_scope[0::2], inst.bin_scope[1::2]
    off = sum(int(inst.dom[bx[k]]) for k in range(c)) * W
    dx, dy = int(inst.dom[bx[c]]), int(inst.dom[by[c]])
    m = np.zeros((dx, dy), bool)
    for a in range(dx):
        m[a] = _bits(inst.bin_rows[off + a * W: off + (a + 1) * W], dy)
    return m if first else m.T


def _expected(inst, x, c1, c2):
    bx, by = inst.bin_scope[0::2], inst.bin_scope[1::2]
    W = inst.W
    y = int(by[c1]) if int(bx[c1]) == x else int(bx[c1])
    z = int(by[c2]) if int(bx[c2]) == y else int(bx[c2])
    dy, dz = int(inst.dom[y]), int(inst.dom[z])
    r1 = _rows(inst, c1, int(bx[c1]) == x)          # [dx, dy]
    r2 = _rows(inst, c2, int(bx[c2]) == z)          # [dz, dy]
    Dy = _bits(inst.init[y * W:(y + 1) * W], dy)
    Dz = _bits(inst.init[z * W:(z + 1) * W], dz)
    cnt = (r1 & Dy).astype(np.int32) @ r2.T.astype(np.int32)   # [dx, dz]
    gone = (cnt == 0) & Dz
    out = np.zeros((128, 2), np.uint64)
    for a in range(r1.shape[0]):
        for v in np.nonzero(gone[a])[0]:
            out[a, v >> 6] |= np.uint64(1) << np.uint64(v & 63)
    return out


@pytest.mark.parametrize("args", [(60, 128, 600, 0.4, 0.4, 0.0, 7),    # W = 2, loose: few removals
                                  (60, 128, 300, 0.93, 0.93, 0.2, 3),  # W = 2, tight: many removals
                                  (50, 64, 300, 0.85, 0.85, 0.1, 5),   # W = 1
                                  (40, 50, 200, 0.8, 0.8, 0.2, 2)])    # W = 1, ragged word
def test_tensor_tiles_equal_bitwise_and_numpy(engine, args):
    inst = cp.gen_binary(*args)
    net = engine.upload(inst)
    tx, t1, t2 = cp.sac_tile_list(inst, range(inst.n), limit=3000)
    assert len(tx) > 500
    bit, _ = net.sac_tiles(tx, t1, t2, mode=0)
    ten, _ = net.sac_tiles(tx, t1, t2, mode=1)
    assert np.array_equal(bit, ten), np.argwhere(bit != ten)[:5]
    if args[3] > 0.8:
        assert bit.any()
    for i in range(0, len(tx), max(1, len(tx) // 25)):
        assert np.array_equal(bit[i], _expected(inst, int(tx[i]), int(t1[i]), int(t2[i]))), i
    net.close()


def test_tensor_tiles_repeat(engine):
    """Two calls in a row (tensor memory and the mbarrier phase reused)."""
    inst = cp.gen_binary(60, 128, 600, 0.9, 0.9, 0.0, 11)
    net = engine.upload(inst)
    tx, t1, t2 = cp.sac_tile_list(inst, range(10))
    a, _ = net.sac_tiles(tx, t1, t2, mode=1)
    b, _ = net.sac_tiles(tx, t1, t2, mode=1)
    c, _ = net.sac_tiles(tx, t1, t2, mode=0)
    assert np.array_equal(a, b) and np.array_equal(a, c)
    net.close()
