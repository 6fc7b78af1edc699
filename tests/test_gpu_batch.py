"""GPU: batched construction (pwmgpu_batch_*): every text of a batch must be
bit-identical to pwm's construction of that text alone (oracle, pwm's
wx_ps::compute restated), on the tile engine (the persistent work-queue
kernel: every tile size, tuned sizes, texts of 1..12 levels so 1 to 3 passes
with the waits between a text's passes) and on the warp-pass engine (every
split-pass width), across CUDA-graph replays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _check_all(batch, texts, offsets, levels, orc, tree=True, indices=None):
    for i in (range(len(levels)) if indices is None else indices):
        t = texts[int(offsets[i]):int(offsets[i + 1])]
        L = int(levels[i])
        if t.size == 0:
            continue
        wm = batch.download(i, 0)
        ref = orc.build(t, L, False, "ps")
        for l in range(L):
            assert np.array_equal(np.asarray(wm.bvs()[l]), ref.level(l)), (i, "matrix", l)
        assert wm.zeros() == [int(z) for z in ref.zeros], (i, "zeros")
        if tree:
            wt = batch.download(i, 1)
            rt = orc.build(t, L, True, "ps")
            for l in range(L):
                assert np.array_equal(np.asarray(wt.bvs()[l]), rt.level(l)), (i, "tree", l)


def _edge_batch(dtype, max_levels, seed):
    rng = np.random.default_rng(seed)
    lens = [1, 2, 31, 63, 64, 65, 1000, 16383, 16384, 16385, 32768, 40000, 70001, 0, 5, 129]
    lens += [int(x) for x in rng.integers(1, 120_000, 24)]
    levels = [int(x) for x in rng.integers(1, max_levels + 1, len(lens))]
    parts = [rng.integers(0, 1 << L, n).astype(dtype) for n, L in zip(lens, levels)]
    offsets = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    return np.concatenate(parts), offsets, np.array(levels, dtype=np.uint32)


def _warp_context(pg):
    ctx = pg.Context()
    ctx.set_engine(pg.ENGINE_WARP)
    return ctx


@pytest.mark.parametrize("vpt", [0, 1, 2, 4])
@pytest.mark.parametrize("width,max_levels,tree", [(1, 8, True), (2, 12, True), (4, 12, False), (1, 12, True)])
def test_tile_batch_matches_single_builds(pg, orc, vpt, width, max_levels, tree):
    """Tile engine, every tile size (0: the tuned ones) and key width; texts
    of up to 12 levels take 3 passes, the later ones waiting for the earlier
    ones of their text inside the persistent kernel."""
    torch = _torch()
    dtype = {1: np.uint8, 2: np.uint16, 4: np.uint32}[width]
    texts, offsets, levels = _edge_batch(dtype, max_levels, 40 + vpt + 7 * width + max_levels)
    d = torch.from_numpy(texts.view({1: np.uint8, 2: np.int16, 4: np.int32}[width])).cuda()
    ctx = pg.Context()
    b = pg.Batch(offsets, levels, word_width=width, tree=tree, context=ctx)
    if vpt:
        b.set_tile_vectors(vpt)
    b.build(d.data_ptr())
    b.check()
    _check_all(b, texts, offsets, levels, orc, tree=tree)
    got = {b.tile_vectors(i) for i in range(len(levels))}
    assert got <= {1, 2, 4} and (vpt == 0 or got == {vpt})
    b.build(d.data_ptr())  # graph replay
    b.check()
    _check_all(b, texts, offsets, levels, orc, tree=tree, indices=[3, 9, 20, 33])
    b.free()


def test_tile_batch_tuning_is_cached_per_class(pg, orc):
    """The tile sizes measured for a batch's classes are reused by a second
    batch with the same classes in the same context."""
    torch = _torch()
    texts, offsets, levels = pg.generate_batch(3, 64)
    d = torch.from_numpy(texts).cuda()
    ctx = pg.Context()
    a = pg.Batch(offsets, levels, word_width=1, tree=True, context=ctx)
    a.build(d.data_ptr())
    a.check()
    b = pg.Batch(offsets, levels, word_width=1, tree=True, context=ctx)
    b.build(d.data_ptr())
    b.check()
    assert [a.tile_vectors(i) for i in range(64)] == [b.tile_vectors(i) for i in range(64)]
    small = [i for i in range(64) if offsets[i + 1] - offsets[i] < 300_000][:12]
    _check_all(b, texts, offsets, levels, orc, indices=small)
    a.free()
    b.free()


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_batch_matches_single_builds(pg, orc, k):
    torch = _torch()
    texts, offsets, levels = _edge_batch(np.uint8, 8, 10 + k)
    d = torch.from_numpy(texts).cuda()
    b = pg.Batch(offsets, levels, word_width=1, tree=True, levels_per_pass=k, context=_warp_context(pg))
    b.build(d.data_ptr())
    b.check()
    _check_all(b, texts, offsets, levels, orc)
    # graph replay gives the same structures
    b.build(d.data_ptr())
    b.check()
    _check_all(b, texts, offsets, levels, orc, indices=[3, 9, 20])
    b.free()


def test_wide_symbols_and_deep_levels(pg, orc):
    torch = _torch()
    texts, offsets, levels = _edge_batch(np.uint16, 12, 99)
    d = torch.from_numpy(texts.view(np.int16)).cuda()
    b = pg.Batch(offsets, levels, word_width=2, tree=True, levels_per_pass=2, context=_warp_context(pg))
    b.build(d.data_ptr())
    b.check()
    _check_all(b, texts, offsets, levels, orc)
    b.free()


def test_retuned_pass_width_rebuilds(pg, orc):
    torch = _torch()
    texts, offsets, levels = _edge_batch(np.uint8, 8, 5)
    d = torch.from_numpy(texts).cuda()
    b = pg.Batch(offsets, levels, word_width=1, tree=True, levels_per_pass=1, context=_warp_context(pg))
    b.build(d.data_ptr())
    for k in (3, 2, 4):
        b.set_levels_per_pass(k)
        b.build(d.data_ptr())
        b.check()
        _check_all(b, texts, offsets, levels, orc, indices=[0, 7, 11, 30])
    b.free()


def test_generated_batch(pg, orc):
    torch = _torch()
    texts, offsets, levels = pg.generate_batch(3, 48)
    assert set(np.unique(levels)) <= {3, 8}
    d = torch.from_numpy(texts).cuda()
    b = pg.Batch(offsets, levels, word_width=1, tree=True, levels_per_pass=2)
    b.build(d.data_ptr())
    b.check()
    small = [i for i in range(48) if offsets[i + 1] - offsets[i] < 400_000][:16]
    _check_all(b, texts, offsets, levels, orc, indices=small)
    b.free()


@pytest.mark.parametrize("engine", ["tile", "warp"])
def test_symbol_out_of_range_in_batch(pg, engine):
    torch = _torch()
    texts = np.array([0, 1, 2, 3, 7, 1], dtype=np.uint8)
    offsets = np.array([0, 3, 6], dtype=np.uint64)
    levels = np.array([2, 2], dtype=np.uint32)  # 7 >= 2^2 in the second text
    d = torch.from_numpy(texts).cuda()
    b = pg.Batch(offsets, levels, context=_warp_context(pg) if engine == "warp" else pg.Context())
    b.build(d.data_ptr())
    with pytest.raises(pg.PwmGpuError) as e:
        b.check()
    assert e.value.status == 5
    b.free()
