"""GPU parity of the Huffman-shaped wavelet matrix / tree (wx_huff_* drop-ins)
and of the code builder against pwm's golden vectors (wx_huff_naive, the
reference's own --check oracle for Huffman shapes) and the oracle."""
import numpy as np
import pytest

from conftest import text_from_hex, words_from_hex
from helpers import seeded_text, sha_words

pytestmark = pytest.mark.gpu

DT = {1: np.uint8, 2: np.uint16, 4: np.uint32}


@pytest.mark.parametrize("tree", [False, True])
def test_codes_match_pwm_on_fixtures(pg, golden_fixtures, tree):
    key = ("wt" if tree else "wm") + "_huff"
    for case in golden_fixtures:
        text = text_from_hex(case["text_hex"])
        if text.size == 0:
            continue
        ln, wd, sizes, levels = pg.huffman_codes(text, tree)
        g = case[key]
        assert [int(x) for x in ln] == g["code_len"] and [int(x) for x in wd] == g["code_word"]
        assert [int(x) for x in sizes] == g["level_bits"]


@pytest.mark.parametrize("tree", [False, True])
@pytest.mark.parametrize("cls", ["wx_huff_ps", "wx_huff_pc", "wx_huff_naive"])
def test_fixtures_match_pwm(pg, golden_fixtures, tree, cls):
    key = ("wt" if tree else "wm") + "_huff"
    algo = getattr(pg, cls)(np.uint8, tree)
    for case in golden_fixtures:
        text = text_from_hex(case["text_hex"])
        if text.size == 0:
            continue
        g = case[key]
        ws = algo.compute(text, text.size, 0)
        assert ws.is_huffman_shaped()
        assert [ws.bvs().level_bit_size(l) for l in range(ws.levels())] == g["level_bits"]
        for l in range(ws.levels()):
            assert np.array_equal(np.asarray(ws.bvs()[l]), words_from_hex(g["levels"][l])), (cls, l)
        if not tree:
            assert ws.zeros() == g["zeros"]


@pytest.mark.parametrize("tree", [False, True])
def test_caller_supplied_codes(pg, golden_fixtures, tree):
    """pwm's own code table passed in (the drop-in path of wx_gpu_huff_*)."""
    key = ("wt" if tree else "wm") + "_huff"
    for case in golden_fixtures[:12]:
        text = text_from_hex(case["text_hex"])
        if text.size == 0:
            continue
        g = case[key]
        codes = (np.array(g["code_len"], np.uint64), np.array(g["code_word"], np.uint64))
        ws = pg.wx_huff_ps(np.uint8, tree).compute(text, text.size, 0, codes=codes)
        for l in range(ws.levels()):
            assert np.array_equal(np.asarray(ws.bvs()[l]), words_from_hex(g["levels"][l]))


@pytest.mark.parametrize("tree", [False, True])
def test_seeded_match_pwm(pg, golden_seeded, tree):
    key = ("wt" if tree else "wm") + "_huff"
    for case in golden_seeded:
        if key not in case:
            continue
        text = seeded_text(pg, case)
        g = case[key]
        ln, wd, sizes, levels = pg.huffman_codes(text, tree)
        assert sha_words(ln) == g["code_len_sha256"] and sha_words(wd) == g["code_word_sha256"], case["name"]
        ws = pg.wx_huff_ps(DT[case["width"]], tree).compute(text, text.size, 0)
        assert [ws.bvs().level_bit_size(l) for l in range(ws.levels())] == g["level_bits"]
        assert [sha_words(ws.bvs()[l]) for l in range(ws.levels())] == g["sha256"], case["name"]
        if not tree:
            assert ws.zeros() == g["zeros"]


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_every_pass_width(pg, orc, k):
    ctx = pg.Context()
    ctx.set_pass_levels(k)
    text = pg.generate(pg.GEN_MIX16, 41, 120_001, 2)
    for tree in (False, True):
        ws = pg.wx_huff_ps(np.uint16, tree, context=ctx).compute(text, text.size, 0)
        ref = orc.huff_build(text, tree)
        assert [ws.bvs().level_bit_size(l) for l in range(ws.levels())] == ref.level_bits
        for l in range(ref.levels):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l))
        if not tree:
            assert ws.zeros() == [int(z) for z in ref.zeros]


def test_long_codes_use_wide_keys(pg, orc):
    # Fibonacci-like frequencies give codes longer than 24 bits (64-bit keys)
    fib = [1, 1]
    while len(fib) < 30:
        fib.append(fib[-1] + fib[-2])
    text = np.repeat(np.arange(30, dtype=np.uint8), fib)
    rng = np.random.default_rng(4)
    rng.shuffle(text)
    for tree in (False, True):
        ln, wd, sizes, levels = orc.huff_codes(text, tree)
        assert levels > 24
        ws = pg.wx_huff_pc(np.uint8, tree).compute(text, text.size, 0)
        ref = orc.huff_build(text, tree)
        for l in range(ref.levels):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l))
        if not tree:
            assert ws.zeros() == [int(z) for z in ref.zeros]


def test_codes_longer_than_32_bits(pg, orc):
    """A caller's prefix code with codes up to 47 bits: 64-bit keys (the
    code and its stop bit), narrowed to 32 bits once the levels left fit."""
    nsym = 48
    ln = np.array([i + 1 for i in range(nsym - 1)] + [nsym - 1], np.uint64)  # i ones then a zero; all ones
    wd = np.array([(1 << (i + 1)) - 2 for i in range(nsym - 1)] + [(1 << (nsym - 1)) - 1], np.uint64)
    rng = np.random.default_rng(9)
    text = rng.integers(0, nsym, 200_003).astype(np.uint8)
    levels = int(ln.max())
    counts = np.bincount(text, minlength=nsym)
    sizes = np.array([int(counts[ln > l].sum()) for l in range(levels)], np.uint64)
    for tree in (False, True):
        ws = pg.wx_huff_ps(np.uint8, tree).compute(text, text.size, 0, codes=(ln, wd))
        ref = orc.huff_build(text, tree, codes=(ln, wd, sizes, levels))
        assert ws.levels() == levels == 47
        for l in range(levels):
            assert np.array_equal(np.asarray(ws.bvs()[l]), ref.level(l)), (tree, l)
        if not tree:
            assert ws.zeros() == [int(z) for z in ref.zeros]


def test_single_symbol_text(pg, orc):
    text = np.full(1000, 7, np.uint8)
    for tree in (False, True):
        ws = pg.wx_huff_ps(np.uint8, tree).compute(text, text.size, 0)
        ref = orc.huff_build(text, tree)
        assert ws.levels() == 1 and np.array_equal(np.asarray(ws.bvs()[0]), ref.level(0))
