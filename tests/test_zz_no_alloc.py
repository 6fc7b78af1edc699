"""GPU: the allocation-free rank/select build (pwmgpu_rank_select_build_noalloc)
against the context-based build (pwmgpu_wx_rank_select_blocks).

The allocation-free entry point serves callers that cannot allocate device
memory while they run (graph capture, host frameworks that own all device
buffers, serving loops); its scratch is a fixed array in the library's device
image.  Here it is called through the C ABI on levels of a structure built by
the regular path, twice in a row on different levels (the second call reuses
the scratch the first one left behind), and its blocks must equal the regular
path's bit for bit (integer data: exact equality).  This file is collected
last so that a run stopping at the first failure has run everything else.
"""
import ctypes

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
