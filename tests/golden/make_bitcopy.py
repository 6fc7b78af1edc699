"""Generates tests/golden/bitcopy.json: golden vectors of pwm's copy_bits, the
bit-range copy of its domain-decomposition merge (include/construction/
merge.hpp:19-190).

Run in a checkout that has the pwm source tree (PWM_REFERENCE names it):

    make -C oracle ref REF=$PWM_REFERENCE && python tests/golden/make_bitcopy.py

Two sources, both run through pwm's own copy_bits (oracle/_ref/libpwmref.so):

* the cases of pwm's test/bit_copy.cpp (byte words): the source and initial
  destination vectors and the sequence of copies are read from that file,
  each copy is replayed, and the result must equal the vector the test
  expects after it;
* seeded cases on 64-bit words (as merge_bit_vectors calls it): random
  sources, offsets and lengths covering the aligned and unaligned paths.
"""
import json
import os
import re
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference  # noqa: E402

REF = os.environ.get("PWM_REFERENCE")
OUT = os.path.dirname(os.path.abspath(__file__))


def byte_vector(text):
    """Values of a `std::vector<uint8_t> { 0b..., ... }` initialiser."""
    return [int(v.replace("'", ""), 2) for v in re.findall(r"0b([01']+)", text)]


def test_file_cases(path):
    src_text = open(path).read()
    cases = []
    for m in re.finditer(r"TEST\(BitCopy,\s*(\w+)\)\s*\{(.*?)\n\}", src_text, re.S):
        name, body = m.group(1), m.group(2)
        src = byte_vector(re.search(r"auto const src = std::vector<uint8_t>\s*\{(.*?)\};", body, re.S).group(1))
        dst = byte_vector(re.search(r"auto dst = std::vector<uint8_t>\s*\{(.*?)\};", body, re.S).group(1))
        steps = []
        for call in re.finditer(r"test\((\d+),\s*(\d+),\s*(\d+)\);\s*bit_compare\(dst,\s*std::vector<uint8_t>\s*\{(.*?)\}\);",
                                body, re.S):
            steps.append({"dst_off": int(call.group(1)), "src_off": int(call.group(2)), "len": int(call.group(3)),
                          "expect": byte_vector(call.group(4))})
        cases.append({"name": name, "src": src, "dst": dst, "steps": steps})
    return cases


def main():
    if not REF or not Reference.available():
        sys.exit("set PWM_REFERENCE to the pwm source tree and run `make -C oracle ref REF=$PWM_REFERENCE` first")
    ref = Reference()
    cases = test_file_cases(os.path.join(REF, "test", "bit_copy.cpp"))
    assert cases and all(c["steps"] for c in cases), "no BitCopy cases found"
    for c in cases:  # pwm's copy_bits must give what its own test expects
        src = np.array(c["src"], dtype=np.uint8)
        dst = np.array(c["dst"], dtype=np.uint8)
        for st in c["steps"]:
            ref.copy_bits(dst, src, st["dst_off"], st["src_off"], st["len"])
            assert dst.tolist() == st["expect"], (c["name"], st)
    rng = np.random.default_rng(2017)
    words = []
    for k in range(48):
        nw = int(rng.integers(1, 9))
        src = rng.integers(0, 1 << 63, nw, dtype=np.uint64) * 2 + rng.integers(0, 2, nw, dtype=np.uint64)
        total = 64 * nw
        src_off = int(rng.integers(0, total))
        length = int(rng.integers(0, total - src_off + 1))
        dst_off = int(rng.integers(0, 64 * 4))
        if k % 4 == 0:  # the same alignment in source and destination (pwm's aligned path)
            dst_off = (dst_off // 64) * 64 + src_off % 64
        dst = np.zeros((dst_off + length + 63) // 64 + 1, dtype=np.uint64)
        ref.copy_bits(dst, src, dst_off, src_off, length)
        words.append({"src": [int(x) for x in src], "dst_words": int(dst.size), "dst_off": dst_off,
                      "src_off": src_off, "len": length, "expect": [int(x) for x in dst]})
    with open(os.path.join(OUT, "bitcopy.json"), "w") as f:
        json.dump({"source": "pwm test/bit_copy.cpp (replayed through pwm's copy_bits) and seeded 64-bit cases",
                   "byte_cases": cases, "word_cases": words}, f, indent=1)
    print(len(cases), "byte cases,", len(words), "word cases")


if __name__ == "__main__":
    main()
