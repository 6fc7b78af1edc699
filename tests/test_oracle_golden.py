"""CPU: the oracle restatement against pwm's own outputs (golden vectors made
by tests/golden/make_golden.py from the reference), and against brute force."""
import numpy as np
import pytest

from conftest import text_from_hex, words_from_hex
from helpers import brute_rank, brute_select, seeded_text, sha_u32, sha_words


def test_fixture_count(golden_fixtures):
    # pwm's roundtrip_batch: corner cases, UTF-8 strings, all 256 byte values
    assert len(golden_fixtures) >= 25
    assert any(c["text_hex"] == "" for c in golden_fixtures)


@pytest.mark.parametrize("variant", ["ps", "pc", "naive", "ppc", "dd_ps"])
@pytest.mark.parametrize("tree", [False, True])
def test_fixtures_construction(orc, golden_fixtures, variant, tree):
    key = "wt" if tree else "wm"
    for case in golden_fixtures:
        text = text_from_hex(case["text_hex"])
        s = orc.build(text, 8, tree, variant)
        g = case[key]
        if text.size == 0:
            assert s.levels == 0 and g["levels"] == []
            continue
        for l in range(8):
            assert np.array_equal(s.level(l), words_from_hex(g["levels"][l])), (variant, tree, l)
        if not tree:
            z = [int(x) for x in s.zeros]
            if variant == "ppc":  # pwm's wx_ppc leaves zeros[L-1] at 0
                assert z[:7] == g["zeros"][:7] and z[7] == 0
            else:
                assert z == g["zeros"]


@pytest.mark.parametrize("tree", [False, True])
def test_fixtures_rank_select_blocks(orc, golden_fixtures, tree):
    key = "wt" if tree else "wm"
    for case in golden_fixtures:
        text = text_from_hex(case["text_hex"])
        if text.size == 0:
            continue
        s = orc.build(text, 8, tree, "ps")
        for l, g in enumerate(case[key + "_rank_select"]):
            l0, l12, s0, s1 = orc.rank_select_blocks(s.level(l))
            assert [int(x) for x in l0] == g["l0"]
            assert np.asarray(l12, "<u4").tobytes().hex() == g["l12"]
            assert [int(x) for x in s0] == g["s0"] and [int(x) for x in s1] == g["s1"]


@pytest.mark.parametrize("tree", [False, True])
def test_fixtures_queries(orc, golden_fixtures, tree):
    key = "wt" if tree else "wm"
    for case in golden_fixtures:
        text = text_from_hex(case["text_hex"])
        if text.size == 0:
            continue
        s = orc.build(text, 8, tree, "ps")
        q = orc.query_support(s)
        assert [q.access(i) for i in range(text.size)] == [int(x) for x in text]
        r = case[key + "_rank"]
        got = [q.rank(a, b) for a, b in zip(r["symbol"], r["index"])]
        assert got == r["result"]
        assert got == [brute_rank(text, a, b) for a, b in zip(r["symbol"], r["index"])]
        # select is not pinned by pwm (its tests are disabled and it reads past
        # its sample table on short levels): brute force instead
        for v in np.unique(text)[:20]:
            occ = int(np.count_nonzero(text == v))
            for k in sorted({1, occ, (occ + 1) // 2}):
                assert q.select(int(v), k) == brute_select(text, v, k)


@pytest.mark.parametrize("tree", [False, True])
def test_fixtures_huffman(orc, golden_fixtures, tree):
    key = ("wt" if tree else "wm") + "_huff"
    for case in golden_fixtures:
        text = text_from_hex(case["text_hex"])
        g = case[key]
        ln, wd, sizes, levels = orc.huff_codes(text, tree)
        assert [int(x) for x in ln] == g["code_len"] and [int(x) for x in wd] == g["code_word"]
        if text.size == 0:
            continue
        s = orc.huff_build(text, tree)
        assert s.level_bits == g["level_bits"]
        for l in range(s.levels):
            assert np.array_equal(s.level(l), words_from_hex(g["levels"][l]))
        if not tree:
            assert [int(z) for z in s.zeros] == g["zeros"]


def test_seeded_texts_are_pinned(pg, orc, golden_seeded):
    import hashlib
    for case in golden_seeded:
        text = seeded_text(pg, case)
        assert hashlib.sha256(text.astype(text.dtype.newbyteorder("<")).tobytes()).hexdigest() == case["text_sha256"]
        # the oracle's copy of the generator gives the same text without the GPU library
        mine = orc.generate(case["dist"], case["seed"], case["n"], case["width"], param=case["param"])
        assert np.array_equal(mine, text), case["name"]


@pytest.mark.parametrize("variant", ["ps", "dd_ps"])
@pytest.mark.parametrize("tree", [False, True])
def test_seeded_construction_and_blocks(orc, pg, golden_seeded, tree, variant):
    key = "wt" if tree else "wm"
    for case in golden_seeded:
        text = seeded_text(pg, case)
        L = case["levels"]
        s = orc.build(text, L, tree, variant, threads=5)
        g = case[key]
        assert [sha_words(s.level(l)) for l in range(L)] == g["sha256"], case["name"]
        if not tree:
            assert [int(z) for z in s.zeros] == g["zeros"]
        for l, gb in enumerate(case[key + "_rank_select"]):
            l0, l12, s0, s1 = orc.rank_select_blocks(s.level(l))
            assert sha_u32(l12) == gb["l12_sha256"] and int(l0.size) == gb["n0"]
            assert sha_u32(s0) == gb["s0_sha256"] and sha_u32(s1) == gb["s1_sha256"]


@pytest.mark.parametrize("tree", [False, True])
def test_seeded_huffman(orc, pg, golden_seeded, tree):
    key = ("wt" if tree else "wm") + "_huff"
    for case in golden_seeded:
        if key not in case:
            continue
        text = seeded_text(pg, case)
        ln, wd, sizes, levels = orc.huff_codes(text, tree)
        g = case[key]
        assert sha_words(ln) == g["code_len_sha256"] and sha_words(wd) == g["code_word_sha256"], case["name"]
        s = orc.huff_build(text, tree, (ln, wd, sizes, levels))
        assert s.level_bits == g["level_bits"]
        assert [sha_words(s.level(l)) for l in range(s.levels)] == g["sha256"]
        if not tree:
            assert [int(z) for z in s.zeros] == g["zeros"]


def test_select_matches_brute_force_on_large_levels(orc):
    rng = np.random.default_rng(3)
    for nw, dens in [(4096, 0.5), (4096, 0.01), (20000, 0.9), (1000, 0.3), (32, 0.5)]:
        bits = rng.random(nw * 64) < dens
        words = np.packbits(bits, bitorder="big").view(">u8").astype(np.uint64)
        blocks = orc.rank_select_blocks(words)
        for val in (0, 1):
            pos = np.nonzero(bits == bool(val))[0]
            if pos.size == 0:
                continue
            occ = np.unique(np.concatenate([np.arange(1, pos.size + 1, max(1, pos.size // 500)),
                                            np.arange(8192, pos.size + 1, 8192), [pos.size]])).astype(np.uint64)
            got = orc.select(val, words, occ, blocks)
            smp = blocks[3] if val else blocks[2]
            direct = ((occ - 1) % 8192 == 0) & ((occ - 1) // 8192 < smp.size)
            truth = pos[occ.astype(np.int64) - 1]
            # pwm returns its stored sample for occ = 8192k+1; samples are exact
            # except in the documented block-boundary case, so compare the rest
            assert np.array_equal(got[~direct], truth[~direct])
        idx = rng.integers(0, nw * 64 + 1, 300)
        cs = np.concatenate([[0], np.cumsum(bits)])
        assert np.array_equal(orc.rank1(words, idx, blocks), cs[idx])


def test_oracle_against_reference_directly(orc):
    from oracle.oracle import Reference
    if not Reference.available():
        pytest.skip("pwm reference shim not built here (oracle/_ref)")
    ref = Reference()
    rng = np.random.default_rng(9)
    for width, L in [(1, 3), (2, 13), (4, 18)]:
        dt = {1: np.uint8, 2: np.uint16, 4: np.uint32}[width]
        for n in (1, 64, 1000, 20_001):
            t = rng.integers(0, 1 << L, n).astype(dt)
            for tree in (False, True):
                assert orc.build(t, L, tree, "ps").same_bits(ref.build(t, L, tree, "ps"))


def test_config_texts_are_pinned(orc):
    """The benchmark workloads' texts at full size, from the oracle's copy of
    the generator, hash to the inputs pwm was run on (tests/golden/configs.json)."""
    import hashlib
    import json
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "configs.json")) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        t = orc.generate(c["dist"], c["seed"], c["n"], c["width"], param=c["param"])
        assert hashlib.sha256(t.astype(t.dtype.newbyteorder("<")).tobytes()).hexdigest() == c["text_sha256"], c["name"]


@pytest.mark.parametrize("variant", ["dd_ps", "ppc"])
def test_config_dna_2p26_matches_pwm(orc, variant):
    """The oracle's parallel restatements (the CPU baseline's code) on the
    2^26 DNA-like text against pwm's hashes at that size."""
    import json
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "configs.json")) as f:
        c = next(x for x in json.load(f)["cases"] if x["name"] == "dna4_2p26_l2")
    t = orc.generate(c["dist"], c["seed"], c["n"], c["width"], param=c["param"])
    for tree, key in ((False, "wm"), (True, "wt")):
        s = orc.build(t, c["levels"], tree, variant, threads=8)
        assert [sha_words(s.level(l)) for l in range(s.levels)] == c[key]["sha256"], (variant, key)
        if not tree and variant != "ppc":  # pwm's wx_ppc leaves zeros[L-1] at 0
            assert [int(z) for z in s.zeros] == c[key]["zeros"]
        for l, gb in enumerate(c[key + "_rank_select"]):
            l0, l12, s0, s1 = orc.rank_select_blocks(s.level(l))
            assert sha_u32(l12) == gb["l12_sha256"] and sha_u32(s0) == gb["s0_sha256"] and \
                sha_u32(s1) == gb["s1_sha256"], (variant, key, l)
