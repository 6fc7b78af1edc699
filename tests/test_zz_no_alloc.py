"""GPU: the allocation-free rank/select build (pwmgpu_rank_select_build_noalloc)
against the context-based build (pwmgpu_wx_rank_select_blocks) and against
pwm's own blocks.

The allocation-free entry point serves callers that cannot allocate device
memory while they run (host frameworks that own every device buffer, serving
loops that cannot take an allocator's implicit synchronisation); its scratch
is a fixed array in the library's device image.  Here it is called through
the C ABI on levels of a structure built by the regular path, several times
in a row on different levels (each call reuses the scratch the one before it
left behind), and its blocks must equal the regular path's bit for bit
(integer data: exact equality), and pwm's bin_rank_popcnt /
bin_select_popcnt blocks recorded in tests/golden/seeded.json.  Edge cases: an
empty level and a level of a multiple of 32 words, whose extra zeroed l12
entry must be written over a pre-filled output.  This file is collected last
so that a run stopping at the first failure has run everything else.
"""
import ctypes
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _noalloc_blocks(torch, lib, words_ptr, nwords, stream):
    n0 = nwords // 67108863 + 1
    n12 = nwords // 32 + 1
    ns = nwords * 64 // 8192 + 2
    l0 = torch.full((n0,), -1, dtype=torch.int64, device="cuda")          # must come back cleared
    l12 = torch.full((2 * n12,), -1, dtype=torch.int32, device="cuda")
    s0 = torch.zeros(ns, dtype=torch.int32, device="cuda")
    s1 = torch.zeros(ns, dtype=torch.int32, device="cuda")
    counts = torch.full((3,), -1, dtype=torch.int64, device="cuda")       # must come back cleared
    st = lib.pwmgpu_rank_select_build_noalloc(ctypes.c_void_p(words_ptr), nwords, ctypes.c_void_p(l0.data_ptr()),
                                              ctypes.c_void_p(l12.data_ptr()), ctypes.c_void_p(s0.data_ptr()),
                                              ctypes.c_void_p(s1.data_ptr()), ctypes.c_void_p(counts.data_ptr()),
                                              ctypes.c_void_p(stream))
    assert st == 0, f"status {st}"
    torch.cuda.synchronize()
    c = counts.cpu().numpy().astype(np.uint64)
    return (l0.cpu().numpy().astype(np.uint64), l12.cpu().numpy().view(np.uint32), s0.cpu().numpy().view(np.uint32)[:c[0]],
            s1.cpu().numpy().view(np.uint32)[:c[1]], c)


def test_noalloc_rank_select_matches_context_build():
    torch = _torch()
    import pwm_gb300 as pg
    n, L = 3_000_017, 8                        # levels of 46,876 words: several select samples per level
    text = pg.generate(pg.GEN_ZIPF256, 77, n, 1)
    ds = pg.DeviceStructure(n, 1, L, matrix=True, tree=True, rank_select=True)
    d_text = torch.from_numpy(text).cuda()
    ds.build(d_text.data_ptr())
    ds.check()
    lib = ds.ctx.lib
    stream = torch.cuda.current_stream().cuda_stream
    calls = [(0, 0), (1, 5), (0, 7)]           # consecutive calls on different levels and structures
    for which, level in calls:
        v = ds.view(which)
        nwords = (v.level_bits[level] + 63) // 64
        words_ptr = v.words + 8 * v.level_offset[level]
        got = _noalloc_blocks(torch, lib, words_ptr, nwords, stream)
        l0, l12, s0, s1 = ds.rank_select_blocks(which, level)
        assert np.array_equal(got[0], l0)
        assert np.array_equal(got[1], l12)
        assert np.array_equal(got[2], s0) and np.array_equal(got[3], s1)
        bits = ds.download(which).bvs()[level]
        ones = int(np.unpackbits(np.asarray(bits).astype(">u8").view(np.uint8)).sum())
        assert int(got[4][2]) == ones
    ds.free()


def _sha(a, dtype):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()


def test_noalloc_rank_select_matches_pwm_golden(golden_seeded):
    """Every level of both structures of the seeded Zipf text (2^18 symbols:
    4096 words per level, a multiple of 32, so pwm keeps its extra zeroed
    l12 entry) against pwm's own blocks."""
    torch = _torch()
    import pwm_gb300 as pg
    case = next(c for c in golden_seeded if c["name"] == "zipf256_l8")
    n, L = case["n"], case["levels"]
    text = pg.generate(case["dist"], case["seed"], n, case["width"], param=case["param"])
    assert _sha(text, "<u1") == case["text_sha256"]
    ds = pg.DeviceStructure(n, 1, L, matrix=True, tree=True, rank_select=False)
    d_text = torch.from_numpy(text).cuda()
    ds.build(d_text.data_ptr())
    ds.check()
    lib = ds.ctx.lib
    stream = torch.cuda.current_stream().cuda_stream
    for which, key in ((0, "wm_rank_select"), (1, "wt_rank_select")):
        v = ds.view(which)
        for level in range(L):
            nwords = (v.level_bits[level] + 63) // 64
            assert nwords % 32 == 0
            l0, l12, s0, s1, counts = _noalloc_blocks(torch, lib, v.words + 8 * v.level_offset[level], nwords, stream)
            g = case[key][level]
            assert l0.size == g["n0"] and not l0.any()
            assert l12.size == 2 * g["n12"] and _sha(l12, "<u4") == g["l12_sha256"], (which, level)
            assert int(counts[0]) == g["ns0"] and _sha(s0, "<u4") == g["s0_sha256"], (which, level)
            assert int(counts[1]) == g["ns1"] and _sha(s1, "<u4") == g["s1_sha256"], (which, level)
    ds.free()


def test_noalloc_empty_level():
    """nwords = 0: l0 and l12 hold one zeroed entry each (pwm's empty
    bin_rank_popcnt), no samples, no ones; outputs start pre-filled."""
    torch = _torch()
    import pwm_gb300 as pg
    lib = pg.default_context().lib
    stream = torch.cuda.current_stream().cuda_stream
    dummy = torch.zeros(16, dtype=torch.int64, device="cuda")
    l0, l12, s0, s1, counts = _noalloc_blocks(torch, lib, dummy.data_ptr(), 0, stream)
    assert l0.tolist() == [0]
    assert l12.tolist() == [0, 0]
    assert s0.size == 0 and s1.size == 0
    assert counts.tolist() == [0, 0, 0]


def test_noalloc_rejects_levels_above_the_limit():
    torch = _torch()
    import pwm_gb300 as pg
    lib = pg.default_context().lib
    dummy = torch.zeros(16, dtype=torch.int64, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    too_many = 33423360 + 1
    st = lib.pwmgpu_rank_select_build_noalloc(p, too_many, p, p, p, p, p, None)
    assert st == 1  # PWMGPU_ERR_ARG, nothing enqueued
    assert int(dummy.sum().item()) == 0
