"""GPU: device-resident Huffman-shaped structures (pwmgpu_wx_build_huffman)
and their queries.

pwm builds Huffman-shaped matrices and trees (wx_huff_*) but answers no
queries on them (include/queries/query_support.hpp:43,55,67 print "NOT YET
IMPLEMENTED"), so the queries are pinned by brute force over the text:
access(i) = text[i], rank(c, i) = occurrences of c in text[:i], select(c, k)
= position of the k-th occurrence.  The structures themselves equal the
oracle's (pwm's wx_huff_naive semantics) bit for bit."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = {1: np.uint8, 2: np.uint16, 4: np.uint32}
NONE = np.uint64(0xFFFFFFFFFFFFFFFF)


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def query(pg, ds, which, op, a, b=None):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    out = np.zeros(max(a.size, 1), dtype=np.uint64)
    bp = np.ascontiguousarray(b, dtype=np.uint64).ctypes.data if b is not None else None
    ds.ctx.check(ds.ctx.lib.pwmgpu_wx_query_host(ds.ctx.h, ds.h, which, op, a.ctypes.data, bp, a.size,
                                                 out.ctypes.data))
    return out[:a.size]


def build(pg, torch, text, tree, codes=None, ctx=None):
    d = torch.from_numpy(text.view(np.uint8).copy()).cuda()
    ds = pg.DeviceStructure.huffman(d.data_ptr(), text.size, text.dtype.itemsize, tree=tree, rank_select=True,
                                    codes=codes, context=ctx)
    ds.check()
    return ds


def check_levels(orc, ds, text, tree):
    ref = orc.huff_build(text, tree)
    ws = ds.download(1 if tree else 0)
    assert ws.levels() == ref.levels
    assert [ws.bvs().level_bit_size(l) for l in range(ws.levels())] == ref.level_bits
    for l in range(ref.levels):
        assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), l
    if not tree:
        assert ws.zeros() == [int(z) for z in ref.zeros]


def check_queries(pg, ds, text, tree, rng, nq=20000, exhaustive=False):
    which = 1 if tree else 0
    n = text.size
    t64 = text.astype(np.uint64)
    # access
    pos = np.arange(n, dtype=np.uint64) if exhaustive else rng.integers(0, n, nq).astype(np.uint64)
    assert np.array_equal(query(pg, ds, which, pg.Q_ACCESS, pos), t64[pos.astype(np.int64)])
    assert query(pg, ds, which, pg.Q_ACCESS, [n, n + 5])[0] == NONE
    # rank / select against the occurrence lists (positions of each symbol, ascending)
    order = np.argsort(text, kind="stable")
    syms, first, counts = np.unique(text[order], return_index=True, return_counts=True)
    occ = {int(s): order[f:f + c] for s, f, c in zip(syms, first, counts)}
    ln, _ = ds.codes()
    absent = [c for c in range(min(ln.size + 3, 70000)) if c not in occ][:5]
    cs = rng.choice(np.concatenate([syms.astype(np.uint64), np.array(absent, dtype=np.uint64)]), nq)
    idx = rng.integers(0, n + 3, nq).astype(np.uint64)  # past the end: clamped to the size
    want_rank = np.array([np.searchsorted(occ[int(c)], min(int(i), n)) if int(c) in occ else 0
                          for c, i in zip(cs, idx)], dtype=np.uint64)
    assert np.array_equal(query(pg, ds, which, pg.Q_RANK, cs, idx), want_rank)
    ks = np.array([rng.integers(1, occ[int(c)].size + 2) if int(c) in occ else rng.integers(0, 3) for c in cs],
                  dtype=np.uint64)
    want_sel = np.array([(occ[int(c)][int(k) - 1] if int(c) in occ and 1 <= int(k) <= occ[int(c)].size
                          else (0 if int(k) == 0 else NONE)) for c, k in zip(cs, ks)], dtype=np.uint64)
    assert np.array_equal(query(pg, ds, which, pg.Q_SELECT, cs, ks), want_sel)
    # every occurrence of the rarest and the most frequent symbol
    for s in (syms[np.argmin(counts)], syms[np.argmax(counts)]):
        o = occ[int(s)]
        k = np.arange(1, o.size + 1, dtype=np.uint64)
        assert np.array_equal(query(pg, ds, which, pg.Q_SELECT, np.full(o.size, s, np.uint64), k),
                              o.astype(np.uint64))
        assert np.array_equal(query(pg, ds, which, pg.Q_RANK, np.full(o.size, s, np.uint64), o.astype(np.uint64) + 1),
                              k)


@pytest.mark.parametrize("tree", [False, True])
@pytest.mark.parametrize("case", ["zipf8", "mix16", "dna", "small"])
def test_builder_codes(pg, orc, tree, case):
    torch = torch_cuda()
    rng = np.random.default_rng(["zipf8", "mix16", "dna", "small"].index(case) * 2 + int(tree))
    if case == "zipf8":
        text = pg.generate(pg.GEN_ZIPF256, 5, 300_007, 1)
    elif case == "mix16":
        text = pg.generate(pg.GEN_MIX16, 6, 200_003, 2)
    elif case == "dna":
        text = rng.choice(np.array([0, 1, 2, 3, 200], np.uint8), 100_001, p=[0.3, 0.2, 0.2, 0.29, 0.01])
    else:
        text = np.array([3, 1, 4, 1, 5, 9, 2, 6, 5, 3, 5], np.uint8)
    ds = build(pg, torch, text, tree)
    check_levels(orc, ds, text, tree)
    ln, wd, sizes, levels = pg.huffman_codes(text, tree)
    gl, gw = ds.codes()
    assert np.array_equal(gl, ln) and np.array_equal(gw, wd)
    check_queries(pg, ds, text, tree, rng, exhaustive=text.size <= 100_001)
    ds.free()


@pytest.mark.parametrize("tree", [False, True])
def test_caller_codes_and_wide_symbols(pg, orc, tree):
    """32-bit symbols with a caller's code table (pwm's builder, run on the
    symbols' ranks) and codes for symbols that never occur."""
    torch = torch_cuda()
    rng = np.random.default_rng(21 + tree)
    ranks = np.minimum(rng.geometric(0.01, 150_001) - 1, 999).astype(np.uint16)
    ln, wd, _, _ = pg.huffman_codes(ranks, tree)
    values = np.sort(rng.choice(1 << 20, ln.size, replace=False)).astype(np.uint64)
    text = values[ranks].astype(np.uint32)
    big_len = np.zeros(int(values[-1]) + 1, np.uint64)
    big_word = np.zeros_like(big_len)
    big_len[values] = ln
    big_word[values] = wd
    ds = build(pg, torch, text, tree, codes=(big_len, big_word))
    check_queries(pg, ds, text, tree, rng)
    # the structure equals a build of the ranks with the same codes
    d = build(pg, torch, ranks, tree, codes=(ln, wd))
    for l in range(ds.levels):
        assert np.array_equal(np.asarray(ds.download(int(tree)).bvs()[l]), np.asarray(d.download(int(tree)).bvs()[l]))
    check_levels(orc, d, ranks, tree)
    ds.free()
    d.free()


@pytest.mark.parametrize("tree", [False, True])
def test_long_codes_and_single_symbol(pg, orc, tree):
    torch = torch_cuda()
    fib = [1, 1]
    while len(fib) < 30:
        fib.append(fib[-1] + fib[-2])
    text = np.repeat(np.arange(30, dtype=np.uint8), fib)
    rng = np.random.default_rng(4)
    rng.shuffle(text)
    ds = build(pg, torch, text, tree)
    assert ds.levels > 24
    check_levels(orc, ds, text, tree)
    check_queries(pg, ds, text, tree, rng)
    ds.free()
    one = np.full(1000, 7, np.uint8)
    ds = build(pg, torch, one, tree)
    assert ds.levels == 1
    check_queries(pg, ds, one, tree, rng, exhaustive=True)
    ds.free()


def test_huffman_wx_errors(pg):
    torch = torch_cuda()
    ctx = pg.default_context()
    text = np.arange(100, dtype=np.uint8)
    d = torch.from_numpy(text).cuda()
    h = ctypes.c_void_p()
    both = pg.MATRIX | pg.TREE | pg.RANK_SELECT
    with pytest.raises(pg.PwmGpuError):
        ctx.check(ctx.lib.pwmgpu_wx_build_huffman(ctx.h, ctypes.c_void_p(d.data_ptr()), 100, 1, both, None, None, 0,
                                                  ctypes.byref(h)))
    with pytest.raises(pg.PwmGpuError):  # a symbol without a code
        ln = np.ones(50, np.uint64)
        pg.DeviceStructure.huffman(d.data_ptr(), 100, 1, codes=(ln, np.arange(50, dtype=np.uint64)))
    ds = pg.DeviceStructure.huffman(d.data_ptr(), 100, 1, tree=True)
    with pytest.raises(pg.PwmGpuError):  # plain builds refuse it
        ds.build(d.data_ptr())
    with pytest.raises(pg.PwmGpuError):  # the tree's wx holds no matrix
        ds.view(0)
    ds.free()
