"""GPU: host-to-host builds (pwmgpu_wx_compute_host, pwmgpu_wx_build_host,
pwmgpu_compute).  A pinned host text is uploaded in pieces that the
histogram follows, and pinned outputs receive each level group as its pass
completes; pageable buffers take one copy each way.  Every combination gives
the oracle's structures bit for bit, and the same words as a build from a
device text followed by pwmgpu_wx_download."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = {1: np.uint8, 2: np.uint16, 4: np.uint32}


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def host_u64(torch, count, pinned):
    t = torch.zeros(max(count, 1), dtype=torch.int64)
    return t.pin_memory() if pinned else t


def host_text(torch, text, pinned):
    t = torch.from_numpy(text.view(np.uint8).copy())
    return t.pin_memory() if pinned else t


def level_words(words, view, l):
    off = int(view.level_offset[l])
    return words[off:off + (int(view.level_bits[l]) + 63) // 64]


def check_against_oracle(orc, text, L, wm_words, zeros, wt_words, vm, vt):
    for tree, words, view in ((False, wm_words, vm), (True, wt_words, vt)):
        if words is None:
            continue
        ref = orc.build(text, L, tree, "ps")
        for l in range(L):
            assert np.array_equal(level_words(words, view, l), ref.level(l)), (tree, l)
        if not tree:
            assert [int(z) for z in zeros] == [int(z) for z in ref.zeros]


@pytest.fixture(scope="module")
def contexts(pg):
    torch_cuda()
    tile = pg.Context()
    tile.set_upload_piece_bytes(1 << 20)  # several pieces per text
    warp = pg.Context()
    warp.set_engine(pg.ENGINE_WARP)
    warp.set_upload_piece_bytes(1 << 20)
    return {"tile": tile, "warp": warp}


CASES = [  # (width, levels, symbols): the histogram writes level 0 for levels <= 8
    (1, 8, 5_000_003),
    (1, 3, 2_100_001),
    (2, 8, 1_700_021),
    (2, 11, 1_300_007),
    (4, 6, 900_001),
    (4, 13, 700_003),
]


@pytest.mark.parametrize("engine", ["tile", "warp"])
@pytest.mark.parametrize("width,L,n", CASES)
@pytest.mark.parametrize("pin_in,pin_out", [(True, True), (True, False), (False, True)])
def test_compute_host_matches_oracle(pg, orc, contexts, engine, width, L, n, pin_in, pin_out):
    torch = torch_cuda()
    ctx = contexts[engine]
    rng = np.random.default_rng(width * 100 + L)
    text = rng.integers(0, 1 << L, n).astype(DT[width])
    ds = pg.DeviceStructure(n, width, L, matrix=True, tree=True, rank_select=True, context=ctx)
    vm, vt = ds.view(0), ds.view(1)
    wm = host_u64(torch, vm.total_words, pin_out)
    wt = host_u64(torch, vt.total_words, pin_out)
    zeros = np.zeros(L, dtype=np.uint64)
    ht = host_text(torch, text, pin_in)
    ds.compute_host(ht.data_ptr(), wm.data_ptr(), zeros, wt.data_ptr())
    wm_np = wm.numpy().view(np.uint64)[:vm.total_words]
    wt_np = wt.numpy().view(np.uint64)[:vt.total_words]
    check_against_oracle(orc, text, L, wm_np, zeros, wt_np, vm, vt)
    # the same words, padding included, as a device-text build and a download
    d = torch.from_numpy(text.view(np.uint8).copy()).cuda()
    ds.build(d.data_ptr())
    ds.check()
    for which, got in ((0, wm_np), (1, wt_np)):
        ref_words = np.zeros(got.size, dtype=np.uint64)
        ctx.check(ctx.lib.pwmgpu_wx_download(ctx.h, ds.h, which, ref_words.ctypes.data_as(pg._lib.u64p), None))
        assert np.array_equal(ref_words, got), which
    # the rank/select support of the host-to-host build answers queries
    idx = rng.integers(0, n, 5000).astype(np.uint64)
    out = np.zeros(5000, dtype=np.uint64)
    ds.compute_host(ht.data_ptr(), None, None, None)
    ctx.check(ctx.lib.pwmgpu_wx_query_host(ctx.h, ds.h, 0, pg.Q_ACCESS, idx.ctypes.data, None, idx.size,
                                           out.ctypes.data))
    assert np.array_equal(out, text[idx.astype(np.int64)].astype(np.uint64))
    ds.free()


@pytest.mark.parametrize("tree_only", [False, True])
def test_single_structure_outputs(pg, orc, contexts, tree_only):
    torch = torch_cuda()
    ctx = contexts["tile"]
    rng = np.random.default_rng(11)
    n, L = 3_333_333, 8
    text = rng.integers(0, 256, n).astype(np.uint8)
    ds = pg.DeviceStructure(n, 1, L, matrix=not tree_only, tree=True, context=ctx)
    vt = ds.view(1)
    wt = host_u64(torch, vt.total_words, True)
    ds.compute_host(host_text(torch, text, True).data_ptr(), None, None, wt.data_ptr())
    check_against_oracle(orc, text, L, None, None, wt.numpy().view(np.uint64), None, vt)
    if not tree_only:
        vm = ds.view(0)
        wm = host_u64(torch, vm.total_words, True)
        zeros = np.zeros(L, dtype=np.uint64)
        ds.compute_host(host_text(torch, text, True).data_ptr(), wm.data_ptr(), zeros, None)
        check_against_oracle(orc, text, L, wm.numpy().view(np.uint64), zeros, None, vm, None)
    else:
        with pytest.raises(pg.PwmGpuError):
            ds.compute_host(host_text(torch, text, True).data_ptr(), wt.data_ptr(), None, None)
    ds.free()


def test_build_host_pinned_pieces(pg, orc, contexts):
    torch = torch_cuda()
    ctx = contexts["tile"]
    rng = np.random.default_rng(12)
    for n in (1, 63, 64, 65, 262_143, 262_144, 262_145, 4_194_305):
        text = rng.integers(0, 256, n).astype(np.uint8)
        ds = pg.DeviceStructure(n, 1, 8, matrix=True, tree=True, context=ctx)
        ds.build_host(host_text(torch, text, True).data_ptr())
        ds.check()
        for which, tree in ((0, False), (1, True)):
            ws = ds.download(which)
            ref = orc.build(text, 8, tree, "ps")
            for l in range(8):
                assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (n, tree, l)
            if not tree:
                assert ws.zeros() == [int(z) for z in ref.zeros]
        ds.free()


def test_drop_in_compute_pinned(pg, orc, contexts):
    """pwmgpu_compute (the drop-in's host path) with pinned text and output."""
    torch = torch_cuda()
    ctx = contexts["tile"]
    rng = np.random.default_rng(13)
    n, L = 2_500_001, 7
    text = rng.integers(0, 1 << L, n).astype(np.uint8)
    ht = host_text(torch, text, True)
    for tree in (False, True):
        ds = pg.DeviceStructure(n, 1, L, matrix=not tree, tree=tree, context=ctx)
        v = ds.view(1 if tree else 0)
        out = host_u64(torch, v.total_words, True)
        zeros = np.zeros(L, dtype=np.uint64)
        ctx.check(ctx.lib.pwmgpu_compute(ctx.h, ht.data_ptr(), n, 1, L, int(tree),
                                         ctypes.cast(out.data_ptr(), pg._lib.u64p),
                                         zeros.ctypes.data_as(pg._lib.u64p)))
        words = out.numpy().view(np.uint64)
        check_against_oracle(orc, text, L, None if tree else words, zeros, words if tree else None,
                             None if tree else v, v if tree else None)
        ds.free()


@pytest.mark.parametrize("chunks", [1, 3, 16])
@pytest.mark.parametrize("width,L,n", [(1, 8, 4_500_007), (1, 5, 3_000_001), (2, 8, 1_100_003), (1, 8, 100_003)])
def test_stream_chunks(pg, orc, width, L, n, chunks):
    """Passes launched in chunks whose finished words stream back (or, for
    texts too small to chunk, whole) give the same structures."""
    torch = torch_cuda()
    ctx = pg.Context()
    ctx.set_upload_piece_bytes(1 << 20)
    ctx.set_stream_chunks(chunks)
    rng = np.random.default_rng(chunks * 7 + L)
    g = np.minimum(rng.geometric(0.02, n) - 1, (1 << L) - 1)
    text = np.where(rng.random(n) < 0.7, g, rng.integers(0, 1 << L, n)).astype(DT[width])
    ds = pg.DeviceStructure(n, width, L, matrix=True, tree=True, rank_select=True, context=ctx)
    vm, vt = ds.view(0), ds.view(1)
    wm = host_u64(torch, vm.total_words, True)
    wt = host_u64(torch, vt.total_words, True)
    wm.fill_(-1)  # every word, padding included, must be written
    wt.fill_(-1)
    zeros = np.zeros(L, dtype=np.uint64)
    ds.compute_host(host_text(torch, text, True).data_ptr(), wm.data_ptr(), zeros, wt.data_ptr())
    wm_np = wm.numpy().view(np.uint64)[:vm.total_words]
    wt_np = wt.numpy().view(np.uint64)[:vt.total_words]
    check_against_oracle(orc, text, L, wm_np, zeros, wt_np, vm, vt)
    for which, got in ((0, wm_np), (1, wt_np)):
        ref_words = np.zeros(got.size, dtype=np.uint64)
        ctx.check(ctx.lib.pwmgpu_wx_download(ctx.h, ds.h, which, ref_words.ctypes.data_as(pg._lib.u64p), None))
        assert np.array_equal(ref_words, got), which
    ds.free()
    with pytest.raises(pg.PwmGpuError):
        ctx.set_stream_chunks(0)
    with pytest.raises(pg.PwmGpuError):
        ctx.set_stream_chunks(17)
    ctx.close()
