"""GPU: mixed query batches (pwmgpu_wx_query_batch_host) answer each query
as the single-kind calls do (pwm's query_support, include/queries/
query_support.hpp:39-178), and access answers equal the text."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def single_kind(ds, which, op, a, b):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    out = np.zeros(max(a.size, 1), dtype=np.uint64)
    ds.ctx.check(ds.ctx.lib.pwmgpu_wx_query_host(ds.ctx.h, ds.h, which, op, a.ctypes.data, b.ctypes.data, a.size,
                                                 out.ctypes.data))
    return out[:a.size]


@pytest.mark.parametrize("dtype,L", [(np.uint8, 8), (np.uint16, 12), (np.uint32, 20)])
def test_mixed_batch_matches_single_kind_calls(pg, dtype, L):
    rng = np.random.default_rng(L)
    n = 70_001
    text = rng.integers(0, 1 << L, n).astype(dtype)
    ds = pg.DeviceStructure(n, text.itemsize, L, matrix=True, tree=True, rank_select=True)
    try:
        ds.build_host(text.ctypes.data)
        ds.check()
        nq = 30_000
        ops = rng.integers(0, 3, nq).astype(np.uint8)
        sym = text[rng.integers(0, n, nq)].astype(np.uint64)
        a = np.where(ops == 0, rng.integers(0, n + 5, nq).astype(np.uint64), sym)  # some accesses past the text
        b = np.where(ops == 1, rng.integers(0, n + 1, nq).astype(np.uint64),
                     rng.integers(1, 40, nq).astype(np.uint64))  # some selects past the last occurrence
        for which in (0, 1):
            got = ds.query_batch_host(which, ops, a, b)
            for op in range(3):
                k = ops == op
                assert np.array_equal(got[k], single_kind(ds, which, op, a[k], b[k])), (which, op)
            acc = (ops == 0) & (a < n)
            assert np.array_equal(got[acc], text[a[acc].astype(np.int64)].astype(np.uint64))
        # accesses alone need no second operand
        idx = rng.integers(0, n, 1000).astype(np.uint64)
        assert np.array_equal(ds.query_batch_host(0, np.zeros(1000, np.uint8), idx),
                              text[idx.astype(np.int64)].astype(np.uint64))
    finally:
        ds.free()


def test_mixed_batch_rejects_bad_kinds_and_missing_operands(pg):
    text = np.arange(1000, dtype=np.uint8)
    ds = pg.DeviceStructure(text.size, 1, 8, matrix=True, rank_select=True)
    try:
        ds.build_host(text.ctypes.data)
        a = np.zeros(4, np.uint64)
        with pytest.raises(pg.PwmGpuError):
            ds.query_batch_host(0, np.array([0, 1, 3, 0], np.uint8), a, a)
        with pytest.raises(pg.PwmGpuError):
            ds.query_batch_host(0, np.array([0, 1, 0, 0], np.uint8), a)  # a rank without b
        assert ds.query_batch_host(0, np.zeros(0, np.uint8), np.zeros(0, np.uint64)).size == 0
    finally:
        ds.free()
