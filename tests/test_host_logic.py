"""CPU: the library's pure C++ host logic, compiled on its own
(tests/host_logic/harness.cpp):

* the Huffman code tables (pwm_gb300/csrc/host_huffman.hpp: pwm's histogram
  order and canonical_huff_codes, include/huffman/huff_codes.hpp:140-285)
  equal pwm's own tables on the golden fixtures (8-bit) and, by hash, on the
  seeded 16-bit texts;
* the streaming tracker (pwm_gb300/csrc/host_stream.hpp) reports every word
  of a level exactly once, and only once all its bits are written."""
import os
import subprocess

import numpy as np
import pytest

from conftest import text_from_hex
from helpers import seeded_text, sha_words

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "host_logic", "harness.cpp")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("host_logic") / "harness")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-o", exe, SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def codes(harness, text, tree):
    t = np.asarray(text)
    nsym = 1 << (8 * t.dtype.itemsize)
    count = np.bincount(t.astype(np.int64), minlength=nsym)
    first = np.full(nsym, (1 << 64) - 1, dtype=np.uint64)
    syms, idx = np.unique(t, return_index=True)
    first[syms.astype(np.int64)] = idx
    inp = "%d\n" % nsym + "".join("%d %d\n" % (int(c), int(f)) for c, f in zip(count, first))
    r = subprocess.run([harness, "huff", str(int(tree)), str(t.dtype.itemsize)], input=inp, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    levels = int(lines[0])
    sizes = [int(x) for x in lines[1].split()]
    pairs = [tuple(int(v) for v in ln.split()) for ln in lines[2:] if ln.strip()]
    return levels, sizes, [p[0] for p in pairs], [p[1] for p in pairs]


@pytest.mark.parametrize("tree", [False, True])
def test_code_tables_match_pwm_fixtures(harness, golden_fixtures, tree):
    key = ("wt" if tree else "wm") + "_huff"
    for case in golden_fixtures:
        text = text_from_hex(case["text_hex"])
        if text.size == 0:
            continue
        levels, sizes, ln, wd = codes(harness, text, tree)
        g = case[key]
        assert ln == g["code_len"] and wd == g["code_word"]
        assert sizes == g["level_bits"] and levels == len(g["level_bits"])


@pytest.mark.parametrize("tree", [False, True])
def test_code_tables_match_pwm_seeded(pg, harness, golden_seeded, tree):
    key = ("wt" if tree else "wm") + "_huff"
    for case in golden_seeded:
        if key not in case:
            continue
        text = seeded_text(pg, case)
        levels, sizes, ln, wd = codes(harness, text, tree)
        g = case[key]
        assert sha_words(np.array(ln, np.uint64)) == g["code_len_sha256"], case["name"]
        assert sha_words(np.array(wd, np.uint64)) == g["code_word_sha256"], case["name"]
        assert sizes == g["level_bits"], case["name"]


def test_stream_tracker(harness):
    r = subprocess.run([harness, "lc", "2024", "3000"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
