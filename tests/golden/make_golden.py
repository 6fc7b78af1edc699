"""Generates the golden vectors under tests/golden/ from kurpicz/pwm itself.

Run in a checkout that has the pwm source tree (default /root/reference,
override with PWM_REFERENCE):

    make -C oracle ref && python tests/golden/make_golden.py

It loads oracle/_ref/libpwmref.so (pwm's own headers behind an extern "C"
shim) and records, for

* every fixture string of pwm's test suite (test::roundtrip_batch in
  test/util/util.hpp, extracted by running that function), and
* seeded synthetic texts produced by pwm_gb300.generate (host generator),

the wavelet matrix / tree bit vectors and zero counts of wx_ps (cross-checked
against wx_pc, wx_naive and wx_dd_ps), the rank/select blocks of pwm's
bin_rank_popcnt / bin_select_popcnt, 8-bit query answers of query_support,
and the Huffman codes and bit vectors of wx_huff_naive.
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference  # noqa: E402
import pwm_gb300 as pg  # noqa: E402  (host generator only; no GPU needed)

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
    ("dna4_l2", pg.GEN_DNA4, 11, 100_003, 1, 0, 2),
    ("zipf256_l8", pg.GEN_ZIPF256, 12, 1 << 18, 1, 0, 8),
    ("uniform_u8_l8_tail", pg.GEN_UNIFORM, 13, 65_537, 1, 256, 8),
    ("mix16_l16", pg.GEN_MIX16, 14, 1 << 16, 2, 0, 16),
    ("uniform_u32_l20", pg.GEN_UNIFORM, 15, 1 << 15, 4, 1 << 20, 20),
    ("uniform_u16_l11", pg.GEN_UNIFORM, 16, 30_000, 2, 1 << 11, 11),
    ("words_2048k", pg.GEN_UNIFORM, 17, 2048 * 64, 1, 4, 2),
]


def seeded(ref):
    cases = []
    for name, dist, seed, n, width, param, levels in SEEDED:
        text = pg.generate(dist, seed, n, width, param=param)
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


def main():
    if not Reference.available():
        sys.exit("oracle/_ref/libpwmref.so missing: run `make -C oracle ref` where the pwm tree exists")
    ref = Reference()
    fx = fixtures(ref)
    with open(os.path.join(OUT, "fixtures.json"), "w") as f:
        json.dump({"source": "pwm test::roundtrip_batch (test/util/util.hpp), outputs of pwm's wx_ps, "
                             "bin_rank_popcnt/bin_select_popcnt, query_support and wx_huff_naive",
                   "cases": fx}, f)
    sd = seeded(ref)
    with open(os.path.join(OUT, "seeded.json"), "w") as f:
        json.dump({"source": "pwm wx_ps / bin_rank_popcnt / bin_select_popcnt / wx_huff_naive on "
                             "pwm_gb300.generate texts", "cases": sd}, f, indent=1)
    print(f"wrote {len(fx)} fixture cases and {len(sd)} seeded cases")


if __name__ == "__main__":
    main()
