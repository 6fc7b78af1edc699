"""GPU parity of the plain wavelet matrix / tree construction, rank/select
blocks and queries against pwm's golden vectors and the oracle.  Integer
work: every comparison is bit-exact."""
import numpy as np
import pytest

from conftest import text_from_hex, words_from_hex
from helpers import brute_rank, brute_select, seeded_text, sha_u32, sha_words

pytestmark = pytest.mark.gpu

DT = {1: np.uint8, 2: np.uint16, 4: np.uint32}


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def to_device(torch, a):
    if a.dtype == np.uint16:
        return torch.from_numpy(a.view(np.int16)).cuda()
    if a.dtype == np.uint32:
        return torch.from_numpy(a.view(np.int32)).cuda()
    if a.dtype == np.uint64:
        return torch.from_numpy(a.view(np.int64)).cuda()
    return torch.from_numpy(a).cuda()


def assert_same(ws, ref, L, tree):
    assert ws.levels() == L
    for l in range(L):
        assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), f"level {l} (tree={tree})"
    if not tree:
        assert ws.zeros() == [int(z) for z in ref.zeros]


@pytest.mark.parametrize("tree", [False, True])
def test_fixtures_match_pwm(pg, golden_fixtures, tree):
    key = "wt" if tree else "wm"
    for case in golden_fixtures:
        text = text_from_hex(case["text_hex"])
        ws = pg.wx_ps(np.uint8, tree).compute(text, text.size, 8)
        if text.size == 0:
            assert ws.levels() == 0
            continue
        g = case[key]
        for l in range(8):
            assert np.array_equal(np.asarray(ws.bvs()[l]), words_from_hex(g["levels"][l])), (case["text_hex"][:20], l)
        if not tree:
            assert ws.zeros() == g["zeros"]


@pytest.mark.parametrize("tree", [False, True])
def test_seeded_match_pwm(pg, golden_seeded, tree):
    key = "wt" if tree else "wm"
    for case in golden_seeded:
        text = seeded_text(pg, case)
        L = case["levels"]
        ws = pg.wx_pc(DT[case["width"]], tree).compute(text, text.size, L)
        assert [sha_words(ws.bvs()[l]) for l in range(L)] == case[key]["sha256"], case["name"]
        if not tree:
            assert ws.zeros() == case[key]["zeros"]


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_every_pass_width_gives_the_same_bits(pg, orc, k):
    ctx = pg.Context()
    ctx.set_pass_levels(k)
    text = pg.generate(pg.GEN_ZIPF256, 21, 300_001, 1)
    for tree in (False, True):
        ws = pg.wx_ps(np.uint8, tree, context=ctx).compute(text, text.size, 8)
        assert_same(ws, orc.build(text, 8, tree, "ps"), 8, tree)
    t16 = pg.generate(pg.GEN_MIX16, 22, 70_000, 2)
    ws = pg.wx_ps(np.uint16, False, context=ctx).compute(t16, t16.size, 16)
    assert_same(ws, orc.build(t16, 16, False, "ps"), 16, False)


SIZES = [1, 2, 31, 32, 33, 63, 64, 65, 127, 128, 129, 2047, 2048, 2049, 4095, 8191, 8192, 8193, 16383, 16384,
         16385, 32767, 32768, 32769, 65536, 100_003]


@pytest.mark.parametrize("width", [1, 2, 4])
def test_edge_sizes(pg, orc, width):
    rng = np.random.default_rng(100 + width)
    for n in SIZES:
        for L in (1, 2, 3, 5, 8):
            text = rng.integers(0, 1 << L, n).astype(DT[width])
            for tree in (False, True):
                ws = pg.wx_ps(DT[width], tree).compute(text, n, L)
                assert_same(ws, orc.build(text, L, tree, "ps"), L, tree)


def test_all_level_counts(pg, orc):
    rng = np.random.default_rng(7)
    for L in range(1, 25):
        text = rng.integers(0, 1 << L, 20_000).astype(np.uint32)
        for tree in (False, True):
            ws = pg.wx_ps(np.uint32, tree).compute(text, text.size, L)
            assert_same(ws, orc.build(text, L, tree, "ps"), L, tree)


def test_deep_trees_of_tiny_texts(pg, orc):
    # nearly every prefix group of the regrouped tree levels is empty: the
    # device derives the segments of all 2^m groups of each level
    rng = np.random.default_rng(17)
    for L in (17, 20, 24):
        for n in (1, 2, 63, 64, 65, 1000):
            text = rng.integers(0, 1 << L, n).astype(np.uint32)
            for tree in (False, True):
                ws = pg.wx_ps(np.uint32, tree).compute(text, n, L)
                assert_same(ws, orc.build(text, L, tree, "ps"), L, tree)


def test_skewed_and_constant_texts(pg, orc):
    texts = [np.zeros(50_000, np.uint8), np.full(40_000, 255, np.uint8),
             np.repeat(np.arange(256, dtype=np.uint8), 300), np.tile(np.array([0, 255], np.uint8), 30_000)]
    for t in texts:
        for tree in (False, True):
            assert_same(pg.wx_ps(np.uint8, tree).compute(t, t.size, 8), orc.build(t, 8, tree, "ps"), 8, tree)


def test_symbol_out_of_range_is_an_error(pg):
    text = np.array([0, 1, 2, 9], dtype=np.uint8)
    with pytest.raises(pg.PwmGpuError) as e:
        pg.wx_ps(np.uint8, False).compute(text, 4, 3)
    assert e.value.status == 5
    # the context stays usable
    ws = pg.wx_ps(np.uint8, False).compute(text, 4, 4)
    assert ws.levels() == 4


def test_invalid_arguments(pg):
    with pytest.raises(pg.PwmGpuError) as e:
        pg.wx_ps(np.uint8, False).compute(np.zeros(10, np.uint8), 10, 0)
    assert e.value.status == 1
    with pytest.raises(pg.PwmGpuError):
        pg.wx_ps(np.uint8, False).compute(np.zeros(10, np.uint8), 10, 25)


def test_registry_lists_gpu_algorithms(pg):
    names = {a.name() for a in pg.algorithm_list.get_algorithm_list(1)}
    assert {"wm_gpu_ps", "wt_gpu_pc", "wm_gpu_ppc", "wt_gpu_dd_ps", "wm_gpu_huff_ps"} <= names
    text = np.frombuffer(b"abracadabra, banana", dtype=np.uint8)
    for a in pg.algorithm_list.get_algorithm_list(1):
        if a.is_huffman_shaped():
            continue
        ws = a.compute_bitvector(text, text.size, 8)
        assert ws.levels() == 8


# ---- device-resident structures: rank/select + queries ---------------------------

def build_device(pg, torch, text, L, tree_too=True):
    ds = pg.DeviceStructure(text.size, text.dtype.itemsize, L, matrix=True, tree=tree_too, rank_select=True)
    d = to_device(torch, text)
    ds.build(d.data_ptr())
    ds.check()
    return ds


def test_device_build_rank_select_blocks_match_pwm(pg, golden_seeded):
    torch = torch_cuda()
    for case in golden_seeded:
        text = seeded_text(pg, case)
        L = case["levels"]
        ds = build_device(pg, torch, text, L)
        for which, key in ((0, "wm"), (1, "wt")):
            ws = ds.download(which)
            assert [sha_words(ws.bvs()[l]) for l in range(L)] == case[key]["sha256"], (case["name"], key)
            for l, g in enumerate(case[key + "_rank_select"]):
                l0, l12, s0, s1 = ds.rank_select_blocks(which, l)
                assert int(l0.size) == g["n0"] and int(l12.size // 2) == g["n12"], (case["name"], key, l)
                assert sha_u32(l12) == g["l12_sha256"], (case["name"], key, l)
                assert sha_u32(s0) == g["s0_sha256"] and sha_u32(s1) == g["s1_sha256"], (case["name"], key, l)
        ds.free()


def run_queries(torch, ds, which, op, a, b=None):
    da = torch.from_numpy(np.asarray(a, dtype=np.int64)).cuda()
    db = torch.from_numpy(np.asarray(b, dtype=np.int64)).cuda() if b is not None else None
    out = torch.empty_like(da)
    ds.query(which, op, da.data_ptr(), None if db is None else db.data_ptr(), da.numel(), out.data_ptr())
    ds.ctx.sync()
    return out.cpu().numpy().astype(np.uint64)


def test_queries_on_fixtures_match_pwm(pg, golden_fixtures):
    torch = torch_cuda()
    for case in golden_fixtures:
        text = text_from_hex(case["text_hex"])
        if text.size == 0:
            continue
        ds = build_device(pg, torch, text, 8)
        for which, key in ((0, "wm"), (1, "wt")):
            acc = run_queries(torch, ds, which, pg.Q_ACCESS, np.arange(text.size))
            assert np.array_equal(acc, text.astype(np.uint64))
            r = case[key + "_rank"]
            got = run_queries(torch, ds, which, pg.Q_RANK, r["symbol"], r["index"])
            assert [int(x) for x in got] == r["result"]
            syms, occs = [], []
            for v in np.unique(text):
                c = int(np.count_nonzero(text == v))
                for k in sorted({1, c, (c + 1) // 2}):
                    syms.append(int(v))
                    occs.append(k)
            got = run_queries(torch, ds, which, pg.Q_SELECT, syms, occs)
            assert [int(x) for x in got] == [brute_select(text, s, k) for s, k in zip(syms, occs)]
        ds.free()


@pytest.mark.parametrize("width,L,dist,param", [(1, 8, 2, 0), (2, 16, 3, 0), (4, 20, 0, 1 << 20), (1, 2, 1, 0)])
def test_queries_match_oracle(pg, orc, width, L, dist, param):
    torch = torch_cuda()
    n = 200_000
    text = pg.generate(dist, 31, n, width, param=param)
    ds = build_device(pg, torch, text, L)
    rng = np.random.default_rng(5)
    for which, tree in ((0, False), (1, True)):
        s = orc.build(text, L, tree, "ps")
        q = orc.query_support(s)
        idx = rng.integers(0, n, 2000)
        acc = run_queries(torch, ds, which, pg.Q_ACCESS, idx)
        assert np.array_equal(acc, text[idx].astype(np.uint64))
        syms = text[rng.integers(0, n, 1000)].astype(np.int64)
        pos = rng.integers(0, n + 1, 1000)
        got = run_queries(torch, ds, which, pg.Q_RANK, syms, pos)
        assert [int(x) for x in got] == [q.rank(int(a), int(b)) for a, b in zip(syms, pos)]
        counts = np.bincount(text.astype(np.int64), minlength=1 << L)
        occ = np.array([rng.integers(1, counts[s] + 1) for s in syms])
        got = run_queries(torch, ds, which, pg.Q_SELECT, syms, occ)
        exp = [q.select(int(a), int(b)) for a, b in zip(syms, occ)]
        assert [int(x) for x in got] == exp
        assert exp[:50] == [brute_select(text, a, b) for a, b in zip(syms[:50], occ[:50])]
    ds.free()
