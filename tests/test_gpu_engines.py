"""GPU: the two split engines of plain builds (segmented tile passes, the
default, and warp-autonomous passes) against the oracle, bit-exact, over the
cases where their tilings differ: partial tiles, prefix-group segments of
every size (segmented tree-writing passes and matrix-only passes with a
regrouped tree), misaligned segment starts and text pointers, every pass
width, and all key widths."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = {1: np.uint8, 2: np.uint16, 4: np.uint32}
TILE = {1: 16384, 2: 8192, 4: 4096}


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def build(pg, ctx, text, L, tree):
    return pg.wx_ps(text.dtype.type, tree, context=ctx).compute(text, text.size, L)


def check(pg, orc, ctx, text, L, label=""):
    for tree in (False, True):
        ws = build(pg, ctx, text, L, tree)
        ref = orc.build(text, L, tree, "ps")
        assert ws.levels() == L
        for l in range(L):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), f"{label} level {l} tree={tree}"
        if not tree:
            assert ws.zeros() == [int(z) for z in ref.zeros], label


@pytest.fixture(scope="module")
def engines(pg):
    torch_cuda()
    tile = pg.Context()
    warp = pg.Context()
    warp.set_engine(pg.ENGINE_WARP)
    return tile, warp


@pytest.mark.parametrize("width", [1, 2, 4])
def test_partial_and_whole_tiles(pg, orc, engines, width):
    tile, _ = engines
    T = TILE[width]
    rng = np.random.default_rng(width)
    L = {1: 8, 2: 11, 4: 13}[width]
    for n in (1, 2, 15, 16, 17, 31, 32, 33, T - 1, T, T + 1, 3 * T + 7):
        text = rng.integers(0, 1 << L, n).astype(DT[width])
        check(pg, orc, tile, text, L, f"n={n}")


@pytest.mark.parametrize("L", list(range(1, 13)))
def test_every_level_count_u8_u16(pg, orc, engines, L):
    tile, _ = engines
    rng = np.random.default_rng(100 + L)
    width = 1 if L <= 8 else 2
    n = 200_003
    # skewed: a geometric symbol mix leaves some prefix groups empty, some tiny
    g = np.minimum(rng.geometric(0.05, n) - 1, (1 << L) - 1)
    text = np.where(rng.random(n) < 0.5, g, rng.integers(0, 1 << L, n)).astype(DT[width])
    check(pg, orc, tile, text, L, f"L={L}")


def test_segmented_deep_passes_u32(pg, orc, engines):
    # u32 tiles hold 4096 keys: with 6M keys the passes at levels 4 and 8 run
    # one segment per prefix group (tree levels written by the pass), the pass
    # at level 12 does not (regrouped tree levels)
    tile, _ = engines
    rng = np.random.default_rng(7)
    n = 6_000_000
    text = rng.integers(0, 1 << 14, n).astype(np.uint32)
    check(pg, orc, tile, text, 14, "u32 L=14")


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_engines_agree(pg, orc, engines, k):
    tile, warp = engines
    tile.set_pass_levels(k)
    try:
        # 1.1M keys: the pass at level 4 runs one segment per prefix group
        text = pg.generate(pg.GEN_ZIPF256, 40 + k, 1_100_003, 1)
        for tree in (False, True):
            a = build(pg, tile, text, 8, tree)
            b = build(pg, warp, text, 8, tree)
            for l in range(8):
                assert np.array_equal(np.asarray(a.bvs()[l]), np.asarray(b.bvs()[l])), (k, tree, l)
            if not tree:
                assert a.zeros() == b.zeros()
        check(pg, orc, tile, text[:300_000], 8, f"k={k}")
    finally:
        tile.set_pass_levels(0)


def test_segmented_byte_text(pg, orc, engines):
    tile, _ = engines
    text = pg.generate(pg.GEN_ZIPF256, 5, 2_000_001, 1)
    check(pg, orc, tile, text, 8, "zipf 2M")
    t16 = pg.generate(pg.GEN_MIX16, 6, 3_000_001, 2)
    check(pg, orc, tile, t16, 16, "mix16 3M")


@pytest.mark.parametrize("L", [9, 12])
def test_byte_text_with_more_levels_than_bits(pg, orc, engines, L):
    # the top L-8 levels of a byte text are all zero bits
    tile, warp = engines
    text = pg.generate(pg.GEN_ZIPF256, 8, 150_001, 1)
    check(pg, orc, tile, text, L, f"u8 L={L}")
    check(pg, orc, warp, text, L, f"u8 L={L} warp")


def test_constant_and_two_symbol_texts(pg, orc, engines):
    tile, _ = engines
    for text in (np.full(70_000, 0xA5, np.uint8), np.full(50_000, 0, np.uint8),
                 np.tile(np.array([0, 255], np.uint8), 40_000), np.full(33_000, 3, np.uint16)):
        L = 8 if text.dtype == np.uint8 else 9
        check(pg, orc, tile, text, L, f"const {text[:2]}")


def test_misaligned_device_text(pg, orc, engines):
    torch = torch_cuda()
    tile, _ = engines
    rng = np.random.default_rng(3)
    n = 123_457
    host = rng.integers(0, 256, n + 16).astype(np.uint8)
    d = torch.from_numpy(host).cuda()
    for off in (0, 1, 3, 5, 15):
        ds = pg.DeviceStructure(n, 1, 8, matrix=True, tree=True, context=tile)
        ds.build(d.data_ptr() + off)
        ds.check()
        text = host[off:off + n]
        for which, tree in ((0, False), (1, True)):
            ws = ds.download(which)
            ref = orc.build(text, 8, tree, "ps")
            for l in range(8):
                assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (off, tree, l)
        ds.free()


@pytest.mark.parametrize("width,L,n", [(1, 8, 1_000_003), (1, 5, 300_001), (2, 11, 700_001), (2, 16, 400_009),
                                       (4, 13, 250_007), (4, 20, 200_003)])
def test_rebuild_overwrites_every_bit(pg, orc, engines, width, L, n):
    """Levels are not zeroed between builds: a structure first built from a
    text whose every bit is 1 and then rebuilt in place from a random text
    must equal the oracle's structures for the second text, with every
    padding bit and word still zero."""
    torch = torch_cuda()
    tile, _ = engines
    rng = np.random.default_rng(L)
    ones = np.full(n, (1 << L) - 1, dtype=DT[width])
    text = rng.integers(0, 1 << L, n).astype(DT[width])
    ds = pg.DeviceStructure(n, width, L, matrix=True, tree=True, context=tile)
    for t in (ones, text):
        d = torch.from_numpy(t.view(np.uint8).copy()).cuda()
        ds.build(d.data_ptr())
        ds.check()
    for which, tree in ((0, False), (1, True)):
        v = ds.view(which)
        words = np.zeros(v.total_words, dtype=np.uint64)
        zeros = np.zeros(L, dtype=np.uint64)
        tile.check(tile.lib.pwmgpu_wx_download(tile.h, ds.h, which, words.ctypes.data_as(pg._lib.u64p),
                                                zeros.ctypes.data_as(pg._lib.u64p)))
        ref = orc.build(text, L, tree, "ps")
        real = (n + 63) // 64
        for l in range(L):
            off = int(v.level_offset[l])
            end = int(v.level_offset[l + 1]) if l + 1 < L else int(v.total_words)
            assert np.array_equal(words[off:off + real], ref.level(l)), (tree, l)
            assert not words[off + real:end].any(), (tree, l, "padding words")
            if n % 64:
                assert int(words[off + real - 1]) & ((1 << (64 - n % 64)) - 1) == 0, (tree, l, "padding bits")
        if not tree:
            assert [int(z) for z in zeros] == [int(z) for z in ref.zeros]
    ds.free()


@pytest.mark.parametrize("width,L", [(1, 5), (1, 6), (1, 7), (2, 7), (4, 6)])
def test_single_pass_of_all_levels(pg, orc, engines, width, L):
    """Texts of 5..7 levels take one tile pass of all their levels (given
    prefixes, up to 64 runs per level and tile, shared words cleared and set
    by the pass): partial tiles, skewed and uniform symbols, a misaligned
    device text, and the same bits as passes of at most 4 levels."""
    torch = torch_cuda()
    tile, _ = engines
    T = TILE[width]
    rng = np.random.default_rng(width * 10 + L)
    for n in (1, 63, T - 1, T + 1, 5 * T + 33, 400_001):
        g = np.minimum(rng.geometric(0.08, n) - 1, (1 << L) - 1)
        text = np.where(rng.random(n) < 0.6, g, rng.integers(0, 1 << L, n)).astype(DT[width])
        check(pg, orc, tile, text, L, f"n={n}")
    k4 = pg.Context()
    k4.set_pass_levels(4)
    text = rng.integers(0, 1 << L, 300_007).astype(DT[width])
    for tree in (False, True):
        a, b = build(pg, tile, text, L, tree), build(pg, k4, text, L, tree)
        for l in range(L):
            assert np.array_equal(np.asarray(a.bvs()[l]), np.asarray(b.bvs()[l])), (tree, l)
    host = np.concatenate([np.zeros(3, DT[width]), text])
    d = torch.from_numpy(host.view(np.uint8).copy()).cuda()
    ds = pg.DeviceStructure(text.size, width, L, matrix=True, tree=True, context=tile)
    ds.build(d.data_ptr() + 3 * width)
    ds.check()
    for which, tree in ((0, False), (1, True)):
        ws, ref = ds.download(which), orc.build(text, L, tree, "ps")
        for l in range(L):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (which, l)
    ds.free()
