"""Generates the golden vectors under tests/golden/ from kurpicz/pwm itself.

Run in a checkout that has the pwm source tree (PWM_REFERENCE names it):

    make -C oracle ref REF=$PWM_REFERENCE && python tests/golden/make_golden.py [which ...]

`which` is any of fixtures, seeded, configs, alphabet (default: all).  It
loads oracle/_ref/libpwmref.so (pwm's own headers behind an extern "C" shim)
and records, for

* every fixture string of pwm's test suite (test::roundtrip_batch in
  test/util/util.hpp, extracted by running that function), and
* seeded synthetic texts from the shared generator (oracle's orc_generate,
  the same code as pwm_gb300.generate; the GPU library is not loaded),

the wavelet matrix / tree bit vectors and zero counts of wx_ps (cross-checked
against wx_pc, wx_naive and wx_dd_ps), the rank/select blocks of pwm's
bin_rank_popcnt / bin_select_popcnt, 8-bit query answers of query_support,
and the Huffman codes and bit vectors of wx_huff_naive.  `configs` does the
same, as SHA-256 per level, for the texts of the benchmark workloads at their
full sizes (pwm's wx_dd_ps, cross-checked against wx_ps or wx_pc), and
`alphabet` records pwm's reduce_alphabet on seeded texts.
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle, Reference  # noqa: E402

GEN_UNIFORM, GEN_DNA4, GEN_ZIPF256, GEN_MIX16 = 0, 1, 2, 3

OUT = os.path.dirname(os.path.abspath(__file__))


def words_hex(a):
    return np.ascontiguousarray(a, dtype="<u8").tobytes().hex()


def sha(a, dtype="<u8"):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()


def structure_full(s):
    return {"level_bits": s.level_bits, "levels": [words_hex(s.level(l)) for l in range(s.levels)],
            "zeros": None if s.zeros is None else [int(z) for z in s.zeros]}


def structure_hashed(s):
    return {"level_bits": s.level_bits, "sha256": [sha(s.level(l)) for l in range(s.levels)],
            "zeros": None if s.zeros is None else [int(z) for z in s.zeros]}


def rank_select(ref, s, full):
    out = []
    for l in range(s.levels):
        l0, l12, s0, s1 = ref.rank_select_blocks(s.level(l))
        if full:
            out.append({"l0": [int(x) for x in l0], "l12": np.asarray(l12, "<u4").tobytes().hex(),
                        "s0": [int(x) for x in s0], "s1": [int(x) for x in s1]})
        else:
            out.append({"n0": int(l0.size), "l12_sha256": sha(l12, "<u4"), "n12": int(l12.size // 2),
                        "s0_sha256": sha(s0, "<u4"), "s1_sha256": sha(s1, "<u4"), "ns0": int(s0.size),
                        "ns1": int(s1.size)})
    return out


def check_variants(ref, text, levels, tree, base):
    for v in ("pc", "naive", "dd_ps", "pps"):
        assert ref.build(text, levels, tree, v).same_bits(base), f"pwm {v} differs from ps"


def fixtures(ref):
    rng = np.random.default_rng(20240607)
    cases = []
    for t in ref.fixtures():
        case = {"text_hex": t.tobytes().hex(), "levels": 8}
        for tree in (False, True):
            s = ref.build(t, 8, tree, "ps")
            if t.size:
                check_variants(ref, t, 8, tree, s)
            key = "wt" if tree else "wm"
            case[key] = structure_full(s)
            if t.size:
                case[key + "_rank_select"] = rank_select(ref, s, full=True)
                idx = np.arange(t.size, dtype=np.uint64)
                acc = ref.queries(tree, t, 8, 0, idx)
                assert np.array_equal(acc, t.astype(np.uint64))
                syms = rng.integers(0, 256, 64).astype(np.uint64)
                syms[: min(32, t.size)] = t[: min(32, t.size)]
                pos = rng.integers(0, t.size + 1, 64).astype(np.uint64)
                case[key + "_rank"] = {"symbol": [int(x) for x in syms], "index": [int(x) for x in pos],
                                       "result": [int(x) for x in ref.queries(tree, t, 8, 1, syms, pos)]}
            hs, (ln, wd) = ref.huff(t, tree, "naive")
            case[key + "_huff"] = {"code_len": [int(x) for x in ln], "code_word": [int(x) for x in wd],
                                   **structure_full(hs)}
            if tree and t.size:
                for v in ("ps", "pc"):
                    assert ref.huff(t, tree, v)[0].same_bits(hs), f"pwm huff {v} tree differs"
        cases.append(case)
    return cases


SEEDED = [
    # (name, dist, seed, n, width, param, levels)
    ("dna4_l2", GEN_DNA4, 11, 100_003, 1, 0, 2),
    ("zipf256_l8", GEN_ZIPF256, 12, 1 << 18, 1, 0, 8),
    ("uniform_u8_l8_tail", GEN_UNIFORM, 13, 65_537, 1, 256, 8),
    ("mix16_l16", GEN_MIX16, 14, 1 << 16, 2, 0, 16),
    ("uniform_u32_l20", GEN_UNIFORM, 15, 1 << 15, 4, 1 << 20, 20),
    ("uniform_u16_l11", GEN_UNIFORM, 16, 30_000, 2, 1 << 11, 11),
    ("words_2048k", GEN_UNIFORM, 17, 2048 * 64, 1, 4, 2),
]


def seeded(ref):
    cases = []
    for name, dist, seed, n, width, param, levels in SEEDED:
        text = Oracle().generate(dist, seed, n, width, param=param)
        case = {"name": name, "dist": dist, "seed": seed, "n": n, "width": width, "param": param,
                "levels": levels, "text_sha256": sha(text, text.dtype.newbyteorder("<"))}
        for tree in (False, True):
            s = ref.build(text, levels, tree, "ps")
            check_variants(ref, text, levels, tree, s)
            key = "wt" if tree else "wm"
            case[key] = structure_hashed(s)
            case[key + "_rank_select"] = rank_select(ref, s, full=False)
            if width <= 2:
                hs, (ln, wd) = ref.huff(text, tree, "naive")
                case[key + "_huff"] = {"code_len_sha256": sha(ln), "code_word_sha256": sha(wd),
                                       "ncodes": int(ln.size), **structure_hashed(hs)}
        cases.append(case)
    return cases


# The benchmark workloads at their full sizes: (name, dist, seed, n, width,
# param, levels, cross-check variant, huffman)
CONFIGS = [
    ("dna4_2p26_l2", GEN_DNA4, 1, 1 << 26, 1, 0, 2, "ps", False),
    ("zipf256_2p30_l8", GEN_ZIPF256, 1, 1 << 30, 1, 0, 8, "ps", False),
    ("mix16_2p28_l16", GEN_MIX16, 3, 1 << 28, 2, 0, 16, "pc", True),
    ("uniform20_u32_2p26_l20", GEN_UNIFORM, 3, 1 << 26, 4, 1 << 20, 20, "pc", False),
]


def configs(ref, names=None):
    orc = Oracle()
    cases = []
    for name, dist, seed, n, width, param, levels, check, huff in CONFIGS:
        if names and name not in names:
            continue
        text = orc.generate(dist, seed, n, width, param=param)
        case = {"name": name, "dist": dist, "seed": seed, "n": n, "width": width, "param": param,
                "levels": levels, "text_sha256": sha(text, text.dtype.newbyteorder("<")),
                "pwm": f"wx_dd_ps (cross-checked against wx_{check})"}
        for tree in (False, True):
            s = ref.build(text, levels, tree, "dd_ps")
            assert ref.build(text, levels, tree, check).same_bits(s), f"{name}: pwm {check} differs from dd_ps"
            key = "wt" if tree else "wm"
            case[key] = structure_hashed(s)
            case[key + "_rank_select"] = rank_select(ref, s, full=False)
            del s
            if huff:
                hs, (ln, wd) = ref.huff(text, tree, "naive")
                case[key + "_huff"] = {"code_len_sha256": sha(ln), "code_word_sha256": sha(wd),
                                       "ncodes": int(ln.size), **structure_hashed(hs),
                                       "rank_select": rank_select(ref, hs, full=False)}
                del hs
            print(name, key, "done", flush=True)
        cases.append(case)
    return cases


# Seeded texts for pwm's reduce_alphabet: (name, dist, seed, n, width, param);
# 8-bit texts stay below 255 (pwm's table has 255 entries).
ALPHABET = [
    ("u8_uniform_200", GEN_UNIFORM, 21, 300_001, 1, 200),
    ("u8_zipf_sparse", GEN_UNIFORM, 22, 4096, 1, 37),
    ("u16_mix", GEN_MIX16, 23, 1 << 20, 2, 0),
    ("u16_uniform_5000", GEN_UNIFORM, 24, 200_003, 2, 5000),
    ("u32_uniform_2p20", GEN_UNIFORM, 25, 1 << 20, 4, 1 << 20),
    ("u32_uniform_2p30", GEN_UNIFORM, 26, 1 << 19, 4, 1 << 30),
]


def alphabet(ref):
    orc = Oracle()
    cases = []
    for name, dist, seed, n, width, param in ALPHABET:
        text = orc.generate(dist, seed, n, width, param=param)
        if width == 1:
            assert int(text.max()) < 255
        out, max_char = ref.reduce_alphabet(text)
        cases.append({"name": name, "dist": dist, "seed": seed, "n": n, "width": width, "param": param,
                      "text_sha256": sha(text, text.dtype.newbyteorder("<")),
                      "out_sha256": sha(out, out.dtype.newbyteorder("<")), "max_char": int(max_char)})
    return cases


def main():
    if not Reference.available():
        sys.exit("oracle/_ref/libpwmref.so missing: run `make -C oracle ref REF=<pwm tree>` first")
    which = set(sys.argv[1:]) or {"fixtures", "seeded", "configs", "alphabet"}
    ref = Reference()
    if "fixtures" in which:
        fx = fixtures(ref)
        with open(os.path.join(OUT, "fixtures.json"), "w") as f:
            json.dump({"source": "pwm test::roundtrip_batch (test/util/util.hpp), outputs of pwm's wx_ps, "
                                 "bin_rank_popcnt/bin_select_popcnt, query_support and wx_huff_naive",
                       "cases": fx}, f)
        print(f"wrote {len(fx)} fixture cases")
    if "seeded" in which:
        sd = seeded(ref)
        with open(os.path.join(OUT, "seeded.json"), "w") as f:
            json.dump({"source": "pwm wx_ps / bin_rank_popcnt / bin_select_popcnt / wx_huff_naive on "
                                 "texts of the shared seeded generator", "cases": sd}, f, indent=1)
        print(f"wrote {len(sd)} seeded cases")
    if "configs" in which:
        cf = configs(ref)
        with open(os.path.join(OUT, "configs.json"), "w") as f:
            json.dump({"source": "pwm wx_dd_ps (cross-checked against wx_ps / wx_pc), bin_rank_popcnt / "
                                 "bin_select_popcnt and wx_huff_naive on the benchmark workloads' texts at full "
                                 "size (shared seeded generator); SHA-256 of each level's words, little endian",
                       "cases": cf}, f, indent=1)
        print(f"wrote {len(cf)} config cases")
    if "alphabet" in which:
        al = alphabet(ref)
        with open(os.path.join(OUT, "alphabet.json"), "w") as f:
            json.dump({"source": "pwm reduce_alphabet (include/util/alphabet_util.hpp:18-45) on texts of the "
                                 "shared seeded generator", "cases": al}, f, indent=1)
        print(f"wrote {len(al)} alphabet cases")


if __name__ == "__main__":
    main()
