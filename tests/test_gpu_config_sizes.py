"""GPU: bit-exact parity at the workloads' full sizes against pwm itself.

tests/golden/configs.json holds, for the benchmark texts at their configured
sizes (2^26 DNA-like bytes with 2 levels; the 1 GiB Zipf byte text with 8
levels, the exact text the benchmark builds; 2^28 16-bit symbols with 16
levels, plain and Huffman-shaped; 2^26 32-bit symbols over 2^20 values with 20
levels), the SHA-256 of every level of pwm's own wavelet matrix and tree
(wx_dd_ps, cross-checked there against wx_ps or wx_pc), the matrix zero
counts, the hashes of pwm's rank/select blocks of every level, and for the
16-bit text pwm's Huffman codes and wx_huff_naive structures.  Here the
texts are generated on the device, their hashes checked, the structures
built by the tile engine (the benchmark's path) with rank/select, and every
level, zero count and block compared with pwm's: integer data, exact
equality.  The 2^26 DNA-like text is also compared word for word with the
oracle.  As an extra, the warp engine must agree with the tile engine on the
1 GiB text.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN, "configs.json")) as _f:
    CONFIGS = {c["name"]: c for c in json.load(_f)["cases"]}

NP = {1: np.uint8, 2: np.uint16, 4: np.uint32}


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _sha(a, dtype):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()


def _device_text(torch, pg, ctx, case):
    dtype = {1: torch.uint8, 2: torch.int16, 4: torch.int32}[case["width"]]
    t = torch.empty(case["n"], dtype=dtype, device="cuda")
    pg.generate(case["dist"], case["seed"], case["n"], case["width"], param=case["param"], device_ptr=t.data_ptr(),
                context=ctx)
    torch.cuda.synchronize()
    host = t.cpu().numpy().view(NP[case["width"]])
    assert _sha(host, host.dtype.newbyteorder("<")) == case["text_sha256"], "generated text differs from pwm's input"
    return t, host


def _check_structure(ds, which, golden, golden_rs, label):
    ws = ds.download(which)
    assert [ws.bvs().level_bit_size(l) for l in range(ws.levels())] == golden["level_bits"], label
    for l in range(ws.levels()):
        assert _sha(ws.bvs()[l], "<u8") == golden["sha256"][l], f"{label}: level {l} differs from pwm"
    if golden["zeros"] is not None:
        assert ws.zeros() == golden["zeros"], f"{label}: zeros differ from pwm"
    for l, g in enumerate(golden_rs):
        l0, l12, s0, s1 = ds.rank_select_blocks(which, l)
        assert l0.size == g["n0"] and not l0.any(), f"{label}: l0 of level {l}"
        assert l12.size == 2 * g["n12"] and _sha(l12, "<u4") == g["l12_sha256"], f"{label}: l12 of level {l}"
        assert s0.size == g["ns0"] and _sha(s0, "<u4") == g["s0_sha256"], f"{label}: select0 of level {l}"
        assert s1.size == g["ns1"] and _sha(s1, "<u4") == g["s1_sha256"], f"{label}: select1 of level {l}"


@pytest.mark.parametrize("name", list(CONFIGS))
def test_plain_config_matches_pwm(pg, name):
    torch = _torch()
    case = CONFIGS[name]
    ctx = pg.Context()
    t, _ = _device_text(torch, pg, ctx, case)
    n, w, L = case["n"], case["width"], case["levels"]
    ds = pg.DeviceStructure(n, w, L, matrix=True, tree=True, rank_select=True, context=ctx)
    ds.build(t.data_ptr())
    ds.check()
    _check_structure(ds, 0, case["wm"], case["wm_rank_select"], name + " matrix")
    _check_structure(ds, 1, case["wt"], case["wt_rank_select"], name + " tree")
    ds.free()


def test_huffman_config_matches_pwm(pg):
    torch = _torch()
    case = CONFIGS["mix16_2p28_l16"]
    ctx = pg.Context()
    t, host = _device_text(torch, pg, ctx, case)
    for tree, key in ((False, "wm_huff"), (True, "wt_huff")):
        g = case[key]
        codes = pg.huffman_codes(host, tree, ctx)  # pwm's builder, restated by the library
        assert codes[0].size == g["ncodes"]
        assert _sha(codes[0], "<u8") == g["code_len_sha256"] and _sha(codes[1], "<u8") == g["code_word_sha256"]
        ds = pg.DeviceStructure.huffman(t.data_ptr(), case["n"], 2, tree=tree, rank_select=True, codes=codes[:2],
                                        context=ctx)
        ds.check()
        _check_structure(ds, 1 if tree else 0, g, g["rank_select"], "huffman " + key)
        ds.free()


def test_dna_2p26_two_levels_match_oracle(pg, orc):
    torch = _torch()
    case = CONFIGS["dna4_2p26_l2"]
    ctx = pg.Context()
    t, host = _device_text(torch, pg, ctx, case)
    n, L = case["n"], case["levels"]
    ds = pg.DeviceStructure(n, 1, L, matrix=True, tree=True, context=ctx)
    ds.build(t.data_ptr())
    ds.check()
    for which, tree in ((0, False), (1, True)):
        ws = ds.download(which)
        ref = orc.build(host, L, tree, "ps")
        for l in range(L):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (tree, l)
        if not tree:
            assert ws.zeros() == [int(z) for z in ref.zeros]
    ds.free()


class _DeviceArray:
    """__cuda_array_interface__ over a library-owned device buffer."""

    def __init__(self, ptr, count):
        self.__cuda_array_interface__ = {"shape": (count,), "typestr": "<i8", "data": (ptr, False), "version": 3}


def test_engines_agree_on_the_1gib_text(pg):
    torch = _torch()
    case = CONFIGS["zipf256_2p30_l8"]
    tile, warp = pg.Context(), pg.Context()
    warp.set_engine(pg.ENGINE_WARP)
    t, _ = _device_text(torch, pg, tile, case)
    n, L = case["n"], case["levels"]
    a = pg.DeviceStructure(n, 1, L, matrix=True, tree=True, context=tile)
    b = pg.DeviceStructure(n, 1, L, matrix=True, tree=True, context=warp)
    a.build(t.data_ptr())
    b.build(t.data_ptr())
    a.check()
    b.check()
    for which in (0, 1):
        va, vb = a.view(which), b.view(which)
        wa = torch.as_tensor(_DeviceArray(int(va.words), int(va.total_words)), device="cuda")
        wb = torch.as_tensor(_DeviceArray(int(vb.words), int(vb.total_words)), device="cuda")
        assert torch.equal(wa, wb), which
    a.free()
    b.free()
