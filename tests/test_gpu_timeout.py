"""GPU: a bounded device-side wait that runs out.

The tile engine's decoupled look-back waits for the counts of the tiles
before it, each wait bounded by the context's spin limit.  Here the failure
is made on the host: with the test hook pwmgpu_ctx_test_withhold_tile the
look-back pass of an 8-level build is launched without its first tile, so
that tile's counts are never published (a flag that nothing sets) and the
other tiles of its segment wait.  With a limit of a few thousand polls every
wait gives up within milliseconds: the kernel records a timeout in the status
word and returns, the build reports PWMGPU_ERR_TIMEOUT, and the same context
then builds the text correctly (equal to the oracle) once the hook is off.
No GPU fault, trap or hang is involved.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PWMGPU_ERR_TIMEOUT = 4


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_lookback_wait_expires_and_context_recovers(pg, orc):
    torch = _torch()
    ctx = pg.Context()
    n, L = 1_000_003, 8  # two tile passes; the second (levels 4-7) looks back
    text = pg.generate(pg.GEN_UNIFORM, 31, n, 1, param=256)  # every 4-bit group spans several tiles
    d_text = torch.from_numpy(text).cuda()
    torch.cuda.synchronize()
    ds = pg.DeviceStructure(n, 1, L, matrix=True, tree=True, context=ctx)
    lib = ctx.lib
    assert lib.pwmgpu_ctx_set_spin_limit(ctx.h, 4096) == 0
    assert lib.pwmgpu_ctx_test_withhold_tile(ctx.h, 1) == 0
    t0 = time.perf_counter()
    st = lib.pwmgpu_wx_build(ctx.h, ds.h, d_text.data_ptr())  # asynchronous: the check reports
    assert st in (0, PWMGPU_ERR_TIMEOUT), st
    if st == 0:
        st = lib.pwmgpu_wx_check(ctx.h, ds.h)
    elapsed = time.perf_counter() - t0
    assert st == PWMGPU_ERR_TIMEOUT, f"status {st}: {lib.pwmgpu_ctx_last_error(ctx.h)}"
    assert elapsed < 30.0  # the waits ended at the short limit, not the default
    # the context stays usable: hook off, default limit, a correct build
    assert lib.pwmgpu_ctx_test_withhold_tile(ctx.h, 0) == 0
    assert lib.pwmgpu_ctx_set_spin_limit(ctx.h, 0) == 0
    ds.build(d_text.data_ptr())
    ds.check()
    for which, tree in ((0, False), (1, True)):
        ws = ds.download(which)
        ref = orc.build(text, L, tree, "ps")
        for l in range(L):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (tree, l)
        if not tree:
            assert ws.zeros() == [int(z) for z in ref.zeros]
    ds.free()
    ctx.close()
