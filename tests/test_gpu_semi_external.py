"""GPU: semi-external construction (pwmgpu_compute_semi_external; pwm's
semi_in, include/external_memory/semi_in/pc_semi_external.hpp:16-230).

Small device budgets force many pieces; the host arrays must equal the
oracle's structures bit for bit (padding words zero), for every key width,
1 to 20 levels, matrix and/or tree, and the words of an in-memory build."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = {1: np.uint8, 2: np.uint16, 4: np.uint32}
MiB = 1 << 20


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def text_of(rng, n, width, L):
    g = np.minimum(rng.geometric(0.03, n) - 1, (1 << L) - 1)
    return np.where(rng.random(n) < 0.6, g, rng.integers(0, 1 << L, n)).astype(DT[width])


def level_words(n):
    return (((n + 63) // 64) + 15) // 16 * 16


def check(orc, text, L, wm, zeros, wt):
    n = text.size
    lw = level_words(n)
    for tree, words in ((False, wm), (True, wt)):
        if words is None:
            continue
        ref = orc.build(text, L, tree, "ps")
        for l in range(L):
            lv = words[l * lw:(l + 1) * lw]
            assert np.array_equal(lv[:(n + 63) // 64], ref.level(l)), (tree, l)
            assert not lv[(n + 63) // 64:].any(), (tree, l)
        if not tree:
            assert [int(z) for z in zeros] == [int(z) for z in ref.zeros]


@pytest.mark.parametrize("width,L,n,budget", [
    (1, 8, 3_000_017, 4 * MiB),     # 6 pieces
    (1, 2, 1_000_003, 1 * MiB),     # 2^16-symbol pieces
    (1, 5, 777_777, 2 * MiB),
    (2, 11, 1_500_007, 4 * MiB),
    (2, 16, 700_001, 8 * MiB),
    (4, 20, 400_009, 4 * MiB),      # deep levels: runs shorter than a word
])
def test_semi_external_matches_oracle(pg, orc, width, L, n, budget):
    torch_cuda()
    rng = np.random.default_rng(width * 100 + L)
    text = text_of(rng, n, width, L)
    wm = np.full(L * level_words(n), 0xA5A5A5A5A5A5A5A5, np.uint64)  # every word must be written
    wt = wm.copy()
    wm, zeros, wt = pg.compute_semi_external(text, L, device_budget=budget, out=(wm, wt))
    check(orc, text, L, wm, zeros, wt)


@pytest.mark.parametrize("matrix,tree", [(True, False), (False, True)])
def test_semi_external_one_structure(pg, orc, matrix, tree):
    torch_cuda()
    rng = np.random.default_rng(7)
    n, L = 1_234_567, 8
    text = text_of(rng, n, 1, L)
    wm, zeros, wt = pg.compute_semi_external(text, L, matrix=matrix, tree=tree, device_budget=2 * MiB)
    assert (wm is None) != matrix and (wt is None) != tree
    check(orc, text, L, wm, zeros, wt)


def test_semi_external_equals_in_memory_build(pg):
    """The same words as a host-to-host build held entirely in HBM, from a
    pinned text into pinned arrays."""
    torch = torch_cuda()
    rng = np.random.default_rng(8)
    n, L = 5_000_011, 8
    text = pg.generate(pg.GEN_ZIPF256, 3, n, 1)
    ds = pg.DeviceStructure(n, 1, L, matrix=True, tree=True)
    vm, vt = ds.view(0), ds.view(1)
    ref_m = np.zeros(vm.total_words, np.uint64)
    ref_t = np.zeros(vt.total_words, np.uint64)
    ref_z = np.zeros(L, np.uint64)
    ds.compute_host(text.ctypes.data, ref_m.ctypes.data, ref_z, ref_t.ctypes.data)
    pin_text = torch.from_numpy(text.copy()).pin_memory()
    ctx = pg.Context()
    # twice (the second call reuses the context's piece buffers and shards),
    # then again after the context released them
    for release in (False, False, True):
        if release:
            ctx.release_scratch()
        out_m = torch.zeros(vm.total_words, dtype=torch.int64).pin_memory()
        out_t = torch.zeros(vt.total_words, dtype=torch.int64).pin_memory()
        _, zeros, _ = pg.compute_semi_external(pin_text.numpy(), L, device_budget=8 * MiB, out=(out_m, out_t),
                                               context=ctx)
        assert np.array_equal(out_m.numpy().view(np.uint64), ref_m)
        assert np.array_equal(out_t.numpy().view(np.uint64), ref_t)
        assert np.array_equal(zeros, ref_z)
    ctx.close()
    ds.free()
    del rng


def test_semi_external_edges(pg, orc):
    torch_cuda()
    # one symbol, a text shorter than a piece, an empty text
    for text, L in ((np.full(300_000, 3, np.uint8), 2), (np.arange(1000, dtype=np.uint16) % 977, 10)):
        wm, zeros, wt = pg.compute_semi_external(text, L, device_budget=4 * MiB)
        check(orc, text, L, wm, zeros, wt)
    wm, zeros, wt = pg.compute_semi_external(np.zeros(0, np.uint8), 4, device_budget=MiB)
    assert not zeros.any()
    with pytest.raises(pg.PwmGpuError):  # below one piece of 2^16 symbols
        pg.compute_semi_external(np.zeros(100_000, np.uint8), 8, device_budget=64 * 1024)
    with pytest.raises(pg.PwmGpuError):  # a symbol >= 2^levels
        pg.compute_semi_external(np.full(200_000, 9, np.uint8), 3, device_budget=MiB)
    with pytest.raises(pg.PwmGpuError):  # no output
        pg.compute_semi_external(np.zeros(10, np.uint8), 3, matrix=False, tree=False)
