"""GPU: host-to-host builds whose pageable text and result arrays are larger
than one pinned staging piece (16 MiB) move through the staging ring, filled
and drained by 1, 3 or the automatic number of host threads, or go to the
driver unstaged (0 threads).  Every way gives the same words as the oracle
(pwm's wx_ps restated) for plain texts and as the unstaged copies for
Huffman-shaped ones.  Integer data: exact equality."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("tree", [False, True])
def test_plain_host_to_host_through_staging(pg, orc, tree):
    _torch()
    n, L = (40 << 20) + 12345, 6  # 2.5 pieces of text, 15 MiB of words per structure + tails
    text = pg.generate(pg.GEN_UNIFORM, 5, n, 1, param=64)
    ref = orc.build(text, L, tree, "ps")
    for threads in (-1, 1, 3, 0):
        ctx = pg.Context()
        ctx.set_host_copy_threads(threads)
        ws = pg.wx_ps(np.uint8, tree, context=ctx).compute(text, n, L)
        for l in range(L):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (threads, l)
        if not tree:
            assert ws.zeros() == [int(z) for z in ref.zeros], threads
        ctx.close()


def test_download_through_staging(pg):
    torch = _torch()
    n, L = (24 << 20) + 3, 12  # 36 MiB of matrix words
    text = pg.generate(pg.GEN_UNIFORM, 8, n, 2, param=1 << 12)
    d = torch.from_numpy(text.view(np.int16)).cuda()
    ctx = pg.Context()
    ds = pg.DeviceStructure(n, 2, L, matrix=True, tree=False, context=ctx)
    ds.build(d.data_ptr())
    ds.check()
    ctx.set_host_copy_threads(0)
    direct = np.asarray(ds.download(0).bvs().data).copy()
    for threads in (-1, 2):
        ctx.set_host_copy_threads(threads)
        assert np.array_equal(np.asarray(ds.download(0).bvs().data), direct), threads
    ds.free()
    ctx.close()


@pytest.mark.parametrize("tree", [False, True])
def test_huffman_host_to_host_through_staging(pg, tree):
    _torch()
    n = (12 << 20) + 777  # 24 MiB of 16-bit text
    text = pg.generate(pg.GEN_MIX16, 4, n, 2)
    ctx = pg.Context()
    codes = pg.huffman_codes(text, tree, ctx)
    ctx.set_host_copy_threads(0)
    a = pg.wx_huff_ps(np.uint16, tree, context=ctx).compute(text, n, 0, codes=codes)
    ctx.set_host_copy_threads(-1)
    b = pg.wx_huff_ps(np.uint16, tree, context=ctx).compute(text, n, 0, codes=codes)
    assert a.levels() == b.levels()
    assert np.array_equal(np.asarray(a.bvs().data), np.asarray(b.bvs().data))
    if not tree:
        assert a.zeros() == b.zeros()
    ctx.close()
