"""CPU: the oracle's restatement of pwm's copy_bits (the bit-range copy of
the domain-decomposition merge) against pwm's own results: the cases of pwm's
test/bit_copy.cpp on byte words and seeded cases on 64-bit words
(tests/golden/bitcopy.json, made by tests/golden/make_bitcopy.py)."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bitcopy.json")


def test_byte_cases_of_pwms_test_file(orc):
    cases = json.load(open(GOLDEN))["byte_cases"]
    assert len(cases) == 3
    for c in cases:
        src = np.array(c["src"], dtype=np.uint8)
        dst = np.array(c["dst"], dtype=np.uint8)
        for st in c["steps"]:
            orc.copy_bits(dst, src, st["dst_off"], st["src_off"], st["len"])
            assert dst.tolist() == st["expect"], (c["name"], st)


def test_seeded_word_cases(orc):
    for c in json.load(open(GOLDEN))["word_cases"]:
        src = np.array(c["src"], dtype=np.uint64)
        dst = np.zeros(c["dst_words"], dtype=np.uint64)
        orc.copy_bits(dst, src, c["dst_off"], c["src_off"], c["len"])
        assert dst.tolist() == c["expect"], c
