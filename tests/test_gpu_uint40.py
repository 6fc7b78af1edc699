"""GPU: texts of pwm's 40-bit symbols (uint40_t, 5 packed little-endian bytes;
pwm registers wm_pc / wt_pc for them, src/register/
sequential_prefix_counting.cpp:16-47).  They are widened to 32 bits on the
device and must give the structures of the same values as 32-bit symbols,
bit for bit the oracle's."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def to_u40(v):
    v = np.asarray(v, dtype=np.uint64)
    b = np.zeros((v.size, 5), np.uint8)
    for k in range(5):
        b[:, k] = ((v >> np.uint64(8 * k)) & np.uint64(0xFF)).astype(np.uint8)
    return b.reshape(-1)


def check(orc, values, L, tree, words, zeros=None):
    ref = orc.build(values.astype(np.uint32), L, tree, "ps")
    lw = ((values.size + 63) // 64 + 15) // 16 * 16
    for l in range(L):
        assert np.array_equal(words[l * lw:l * lw + (values.size + 63) // 64], ref.level(l)), (tree, l)
    if zeros is not None:
        assert [int(z) for z in zeros] == [int(z) for z in ref.zeros]


@pytest.mark.parametrize("L,n", [(12, 1_000_003), (4, 300_001), (20, 200_003)])
def test_drop_in_compute_u40(pg, orc, L, n):
    torch_cuda()
    ctx = pg.default_context()
    rng = np.random.default_rng(L)
    values = rng.integers(0, 1 << L, n).astype(np.uint64)
    text = to_u40(values)
    lw = ((n + 63) // 64 + 15) // 16 * 16
    for tree in (0, 1):
        bv = np.zeros(L * lw, np.uint64)
        zeros = np.zeros(L, np.uint64)
        ctx.check(ctx.lib.pwmgpu_compute(ctx.h, text.ctypes.data, n, 5, L, tree, bv.ctypes.data_as(pg._lib.u64p),
                                         zeros.ctypes.data_as(pg._lib.u64p)))
        check(orc, values, L, bool(tree), bv, None if tree else zeros)


def test_device_builds_u40(pg, orc):
    torch = torch_cuda()
    rng = np.random.default_rng(40)
    n, L = 2_000_003, 10
    values = np.minimum(rng.geometric(0.01, n) - 1, (1 << L) - 1).astype(np.uint64)
    text = to_u40(values)
    d = torch.from_numpy(text).cuda()
    ds = pg.DeviceStructure(n, 5, L, matrix=True, tree=True, rank_select=True)
    for build in (lambda: ds.build(d.data_ptr()), lambda: ds.build_sharded(d.data_ptr(), 3),
                  lambda: ds.build_host(text.ctypes.data)):
        build()
        ds.check()
        for which in (0, 1):
            ws = ds.download(which)
            ref = orc.build(values.astype(np.uint32), L, bool(which), "ps")
            for l in range(L):
                assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (which, l)
    # host to host into pinned arrays, and queries on the result
    vm, vt = ds.view(0), ds.view(1)
    wm = torch.zeros(vm.total_words, dtype=torch.int64).pin_memory()
    wt = torch.zeros(vt.total_words, dtype=torch.int64).pin_memory()
    zeros = np.zeros(L, np.uint64)
    pin = torch.from_numpy(text).pin_memory()
    ds.compute_host(pin.data_ptr(), wm.data_ptr(), zeros, wt.data_ptr())
    check(orc, values, L, False, wm.numpy().view(np.uint64), zeros)
    check(orc, values, L, True, wt.numpy().view(np.uint64))
    idx = rng.integers(0, n, 3000).astype(np.uint64)
    out = np.zeros(idx.size, np.uint64)
    ds.ctx.check(ds.ctx.lib.pwmgpu_wx_query_host(ds.ctx.h, ds.h, 0, pg.Q_ACCESS, idx.ctypes.data, None, idx.size,
                                                 out.ctypes.data))
    assert np.array_equal(out, values[idx.astype(np.int64)])
    ds.free()


def test_u40_rejects_out_of_range(pg):
    torch_cuda()
    ctx = pg.default_context()
    n, L = 100_000, 8
    lw = ((n + 63) // 64 + 15) // 16 * 16
    bv = np.zeros(L * lw, np.uint64)
    zeros = np.zeros(L, np.uint64)
    for bad in (1 << 32, 1 << 8, (1 << 39) + 3):  # past 32 bits, past the levels
        values = np.zeros(n, np.uint64)
        values[n // 2] = bad
        text = to_u40(values)
        st = ctx.lib.pwmgpu_compute(ctx.h, text.ctypes.data, n, 5, L, 0, bv.ctypes.data_as(pg._lib.u64p),
                                    zeros.ctypes.data_as(pg._lib.u64p))
        assert st != 0
    # widths other than 1, 2, 4 and 5 stay invalid; the Huffman and
    # semi-external paths take 1, 2 and 4 only
    st = ctx.lib.pwmgpu_compute(ctx.h, np.zeros(30, np.uint8).ctypes.data, 10, 3, 4, 0,
                                bv.ctypes.data_as(pg._lib.u64p), zeros.ctypes.data_as(pg._lib.u64p))
    assert st != 0
    out = np.zeros(4 * 16, np.uint64)
    st = ctx.lib.pwmgpu_compute_semi_external(ctx.h, np.zeros(50, np.uint8).ctypes.data, 10, 5, 4,
                                              out.ctypes.data_as(pg._lib.u64p), None, None, 0)
    assert st != 0
