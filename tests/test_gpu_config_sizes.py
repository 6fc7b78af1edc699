"""GPU: parity at the workloads' full sizes.  Where the oracle finishes in
seconds (2^26 DNA-like symbols, 2 levels) the structures are compared with it
bit for bit; at 2^30 bytes (8 levels), 2^28 16-bit symbols (16 levels) and
2^26 32-bit symbols (20 levels) through size-independent properties: the two
split engines (each checked against the oracle at smaller sizes) agree bit
for bit on every level of both structures, every sampled access query
returns the text's symbol, and the matrix zero counts equal those of the
text's histogram."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _device_text(torch, pg, ctx, dist, seed, n, width, param=0):
    dtype = {1: torch.uint8, 2: torch.int16, 4: torch.int32}[width]
    t = torch.empty(n, dtype=dtype, device="cuda")
    pg.generate(dist, seed, n, width, param=param, device_ptr=t.data_ptr(), context=ctx)
    torch.cuda.synchronize()
    return t


def _build(pg, ctx, t, n, width, L, tree=True, rank_select=True):
    ds = pg.DeviceStructure(n, width, L, matrix=True, tree=tree, rank_select=rank_select, context=ctx)
    ds.build(t.data_ptr())
    ds.check()
    return ds


def _words(torch, ds, which):
    v = ds.view(which)
    # all level words of the structure as a device tensor (no copy)
    return torch.as_tensor(_DeviceArray(int(v.words), int(v.total_words)), device="cuda")


class _DeviceArray:
    """__cuda_array_interface__ over a library-owned device buffer."""

    def __init__(self, ptr, count):
        # int64 view of the u64 words: equality of bits is all that is asked
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<i8", "data": (ptr, False), "version": 3}


def _levels_equal(torch, a, b, which, L):
    va, vb = a.view(which), b.view(which)
    wa, wb = _words(torch, a, which), _words(torch, b, which)
    for l in range(L):
        na = (int(va.level_bits[l]) + 63) // 64
        oa, ob = int(va.level_offset[l]), int(vb.level_offset[l])
        if not torch.equal(wa[oa:oa + na], wb[ob:ob + na]):
            return l
    return None


def _sampled_access(torch, ds, which, t_host, n, k=20000, seed=0):
    rng = np.random.default_rng(seed)
    idx = rng.integers(0, n, k).astype(np.int64)
    d_idx = torch.from_numpy(idx).cuda()
    out = torch.empty(k, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()  # the library's stream is not torch's
    ds.query(which, 0, d_idx.data_ptr(), None, k, out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.uint64)
    return np.array_equal(got, t_host[idx].astype(np.uint64))


def _zeros_from_hist(hist, L):
    syms = np.arange(1 << L)
    return [int(hist[((syms >> (L - 1 - m)) & 1) == 0].sum()) for m in range(L)]


def test_dna_2p26_two_levels_match_oracle(pg, orc):
    torch = _torch()
    ctx = pg.Context()
    n, L = 1 << 26, 2
    t = _device_text(torch, pg, ctx, pg.GEN_DNA4, 1, n, 1)
    host = t.cpu().numpy()
    ds = _build(pg, ctx, t, n, 1, L, rank_select=False)
    for which, tree in ((0, False), (1, True)):
        ws = ds.download(which)
        ref = orc.build(host, L, tree, "ps")
        for l in range(L):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (tree, l)
        if not tree:
            assert ws.zeros() == [int(z) for z in ref.zeros]
    ds.free()


@pytest.mark.parametrize("n,width,L,dist,param", [
    (1 << 30, 1, 8, 2, 0),          # 1 GiB of Zipf bytes
    (1 << 28, 2, 16, 3, 0),         # 16-bit mixture, 16 levels
    (1 << 26, 4, 20, 0, 1 << 20),   # 32-bit uniform over 2^20, 20 levels
])
def test_full_size_properties(pg, n, width, L, dist, param):
    torch = _torch()
    tile = pg.Context()
    warp = pg.Context()
    warp.set_engine(pg.ENGINE_WARP)
    t = _device_text(torch, pg, tile, dist, 7, n, width, param)
    host = t.cpu().numpy().view({1: np.uint8, 2: np.uint16, 4: np.uint32}[width])
    a = _build(pg, tile, t, n, width, L)
    b = _build(pg, warp, t, n, width, L)
    for which in (0, 1):
        assert _levels_equal(torch, a, b, which, L) is None, which
        assert _sampled_access(torch, a, which, host, n, seed=which)
    hist = np.bincount(host.astype(np.int64), minlength=1 << L)
    v = a.view(0)
    assert [int(v.zeros[m]) for m in range(L)] == _zeros_from_hist(hist, L)
    a.free()
    b.free()
