"""GPU: matrix-only builds of more than 8 levels, which plan their passes from
the counts of each pass's own digit (pass_digits_kernel) instead of a leaf
histogram of 2^L bins.  Every level and zero count must equal pwm's (golden
hashes of pwm's wavelet matrix at the configured sizes, with rank/select
blocks) and the oracle's (pwm's wx_ps restated) on seeded texts of 9..24
levels, 8-, 16- and 32-bit symbols, odd sizes, passes of 1..4 levels.
Integer data: exact equality."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

DT = {1: np.uint8, 2: np.uint16, 4: np.uint32}

with open(os.path.join(GOLDEN, "configs.json")) as _f:
    CONFIGS = {c["name"]: c for c in json.load(_f)["cases"]}


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _sha(a, dtype):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()


@pytest.mark.parametrize("name", ["uniform20_u32_2p26_l20", "mix16_2p28_l16"])
def test_full_size_matrix_only_matches_pwm(pg, name):
    torch = _torch()
    case = CONFIGS[name]
    ctx = pg.Context()
    dtype = {1: torch.uint8, 2: torch.int16, 4: torch.int32}[case["width"]]
    t = torch.empty(case["n"], dtype=dtype, device="cuda")
    pg.generate(case["dist"], case["seed"], case["n"], case["width"], param=case["param"], device_ptr=t.data_ptr(),
                context=ctx)
    ds = pg.DeviceStructure(case["n"], case["width"], case["levels"], matrix=True, tree=False, rank_select=True,
                            context=ctx)
    for _ in range(2):  # the second build reuses the context's buffers
        ds.build(t.data_ptr())
        ds.check()
    ws = ds.download(0)
    g = case["wm"]
    for l in range(ws.levels()):
        assert _sha(ws.bvs()[l], "<u8") == g["sha256"][l], f"level {l} differs from pwm"
    assert ws.zeros() == g["zeros"]
    for l, r in enumerate(case["wm_rank_select"]):
        l0, l12, s0, s1 = ds.rank_select_blocks(0, l)
        assert _sha(l12, "<u4") == r["l12_sha256"] and _sha(s0, "<u4") == r["s0_sha256"], l
        assert _sha(s1, "<u4") == r["s1_sha256"], l
    ds.free()
    ctx.close()


@pytest.mark.parametrize("width,L", [(1, 9), (1, 12), (2, 11), (2, 16), (4, 17), (4, 21), (4, 24)])
@pytest.mark.parametrize("n", [1, 63, 100_003])
def test_matrix_only_deep_matches_oracle(pg, orc, width, L, n):
    _torch()
    rng = np.random.default_rng(width * 1000 + L * 10 + n % 97)
    top = min(1 << L, 1 << (8 * width))
    text = rng.integers(0, top, n, dtype=np.uint64).astype(DT[width])
    ws = pg.wx_ps(DT[width], False).compute(text, n, L)
    ref = orc.build(text, L, False, "ps")
    for l in range(L):
        assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), l
    assert ws.zeros() == [int(z) for z in ref.zeros]


@pytest.mark.parametrize("k", [1, 2, 3])
def test_matrix_only_pass_widths(pg, orc, k):
    _torch()
    rng = np.random.default_rng(77 + k)
    n, L = 200_001, 13
    text = (rng.zipf(1.3, n) % (1 << L)).astype(np.uint16)
    ctx = pg.Context()
    ctx.set_pass_levels(k)  # up to 13 passes of one level
    ws = pg.wx_ps(np.uint16, False, context=ctx).compute(text, n, L)
    ref = orc.build(text, L, False, "ps")
    for l in range(L):
        assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), l
    assert ws.zeros() == [int(z) for z in ref.zeros]
    ctx.close()


def test_matrix_only_symbol_out_of_range(pg):
    _torch()
    text = (np.arange(5000) % 1000).astype(np.uint16)
    text[4321] = 1 << 10  # >= 2^10, < 2^11
    ctx = pg.Context()
    with pytest.raises(pg.PwmGpuError) as e:
        pg.wx_ps(np.uint16, False, context=ctx).compute(text, text.size, 10)
    assert e.value.status == 5
    ws = pg.wx_ps(np.uint16, False, context=ctx).compute(text, text.size, 11)  # the context stays usable
    assert ws.levels() == 11
    ctx.close()
