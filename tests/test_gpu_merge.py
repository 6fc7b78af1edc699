"""GPU: the domain-decomposition merge (pwm's wx_dd_ps / wx_dd_pc,
include/construction/merge.hpp) and its bit-range copy.

* pwmgpu_copy_bits against pwm's copy_bits: the cases of pwm's
  test/bit_copy.cpp (byte words, compared as bit sequences) and seeded
  64-bit-word cases (tests/golden/bitcopy.json);
* sharded builds (pwm's slices, merged) equal the oracle's plain build bit
  for bit, matrix zeros included, for shard counts above and below the text
  size, every key width and level counts from 1 to 16;
* shards built by the caller merge into a structure with rank/select that
  answers queries, and merged structures merge again."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = {1: np.uint8, 2: np.uint16, 4: np.uint32}
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bitcopy.json")


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def bits_of_bytes(b):
    return np.unpackbits(np.asarray(b, dtype=np.uint8))  # MSB first within each byte


def words_of_bits(bits):
    """Bit sequence -> uint64 words, bit i at bit 63 - i%64 of word i/64."""
    padded = np.zeros(((bits.size + 63) // 64) * 64, dtype=np.uint8)
    padded[:bits.size] = bits
    return np.packbits(padded).view(">u8").astype(np.uint64)


def test_copy_bits_matches_pwm(pg):
    torch = torch_cuda()
    g = json.load(open(GOLDEN))
    for c in g["byte_cases"]:
        src = torch.from_numpy(words_of_bits(bits_of_bytes(c["src"])).view(np.int64)).cuda()
        dst = torch.from_numpy(words_of_bits(bits_of_bytes(c["dst"])).view(np.int64)).cuda()
        for st in c["steps"]:
            pg.copy_bits(dst.data_ptr(), src.data_ptr(), st["dst_off"], st["src_off"], st["len"])
            torch.cuda.synchronize()
            nbits = 8 * len(st["expect"])
            got = np.unpackbits(dst.cpu().numpy().view(np.uint64).astype(">u8").view(np.uint8))[:nbits]
            assert np.array_equal(got, bits_of_bytes(st["expect"])), (c["name"], st)
    for c in g["word_cases"]:
        src = torch.from_numpy(np.array(c["src"], dtype=np.uint64).view(np.int64)).cuda()
        dst = torch.zeros(c["dst_words"], dtype=torch.int64, device="cuda")
        pg.copy_bits(dst.data_ptr(), src.data_ptr(), c["dst_off"], c["src_off"], c["len"])
        torch.cuda.synchronize()
        assert dst.cpu().numpy().view(np.uint64).tolist() == c["expect"], c


def check_structures(orc, ds, text, L, zeros=True):
    for which, tree in ((0, False), (1, True)):
        ws = ds.download(which)
        ref = orc.build(text, L, tree, "ps")
        for l in range(L):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (tree, l)
        if not tree and zeros:
            assert ws.zeros() == [int(z) for z in ref.zeros]


@pytest.mark.parametrize("width,L", [(1, 8), (1, 3), (1, 1), (2, 11), (2, 16), (4, 13)])
@pytest.mark.parametrize("shards", [2, 3, 7, 16])
def test_sharded_build_matches_oracle(pg, orc, width, L, shards):
    torch = torch_cuda()
    rng = np.random.default_rng(width * 1000 + L * 10 + shards)
    for n in (5, 1000, 300_007):
        g = np.minimum(rng.geometric(0.05, n) - 1, (1 << L) - 1)
        text = np.where(rng.random(n) < 0.5, g, rng.integers(0, 1 << L, n)).astype(DT[width])
        d = torch.from_numpy(text.view(np.uint8).copy()).cuda()
        ds = pg.DeviceStructure(n, width, L, matrix=True, tree=True)
        ds.build_sharded(d.data_ptr(), shards)
        ds.check()
        check_structures(orc, ds, text, L)
        ds.free()


def test_caller_built_shards_merge_with_rank_select(pg, orc):
    torch = torch_cuda()
    rng = np.random.default_rng(5)
    L, n = 8, 1_000_003
    text = pg.generate(pg.GEN_ZIPF256, 9, n, 1)
    cuts = [0, 1, 250_000, 250_000, 777_777, n]  # an empty shard and a one-symbol shard
    parts = []
    for a, b in zip(cuts[:-1], cuts[1:]):
        p = pg.DeviceStructure(b - a, 1, L, matrix=True, tree=True, keep_histogram=True)
        d = torch.from_numpy(text[a:b].copy()).cuda() if b > a else torch.zeros(1, dtype=torch.uint8, device="cuda")
        p.build(d.data_ptr())
        p.check()
        parts.append(p)
    out = pg.DeviceStructure(n, 1, L, matrix=True, tree=True, rank_select=True, keep_histogram=True)
    out.merge(parts)
    check_structures(orc, out, text, L)
    idx = rng.integers(0, n, 4000).astype(np.int64)
    for which in (0, 1):
        da = torch.from_numpy(idx).cuda()
        res = torch.empty_like(da)
        out.query(which, pg.Q_ACCESS, da.data_ptr(), None, idx.size, res.data_ptr())
        out.ctx.sync()
        assert np.array_equal(res.cpu().numpy().astype(np.uint64), text[idx].astype(np.uint64))
    # merged structures merge again: (parts 0-2) + (parts 3-4)
    left = pg.DeviceStructure(cuts[3], 1, L, matrix=True, tree=True, keep_histogram=True)
    left.merge(parts[:3])
    right = pg.DeviceStructure(n - cuts[3], 1, L, matrix=True, tree=True, keep_histogram=True)
    right.merge(parts[3:])
    again = pg.DeviceStructure(n, 1, L, matrix=True, tree=True)
    again.merge([left, right])
    check_structures(orc, again, text, L)
    for x in parts + [out, left, right, again]:
        x.free()


def test_merge_rejects_bad_shards(pg):
    torch = torch_cuda()
    text = np.arange(1000, dtype=np.uint8)
    d = torch.from_numpy(text).cuda()
    no_hist = pg.DeviceStructure(1000, 1, 8, matrix=True, tree=True)
    no_hist.build(d.data_ptr())
    out = pg.DeviceStructure(1000, 1, 8, matrix=True, tree=True)
    with pytest.raises(pg.PwmGpuError):
        out.merge([no_hist])
    ok = pg.DeviceStructure(1000, 1, 8, matrix=True, tree=True, keep_histogram=True)
    ok.build(d.data_ptr())
    bigger = pg.DeviceStructure(1001, 1, 8, matrix=True, tree=True)
    with pytest.raises(pg.PwmGpuError):
        bigger.merge([ok])
    deep = pg.DeviceStructure(1000, 4, 17, matrix=True, tree=False)
    with pytest.raises(pg.PwmGpuError):
        deep.merge([ok])
    for x in (no_hist, out, ok, bigger, deep):
        x.free()
