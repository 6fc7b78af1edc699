"""CPU: the library's pure C++ host logic, compiled on its own
(tests/host_logic/harness.cpp):

* the Huffman code tables (pwm_gb300/csrc/host_huffman.hpp: pwm's histogram
  order and canonical_huff_codes, include/huffman/huff_codes.hpp:140-285)
  equal pwm's own tables on the golden fixtures (8-bit) and, by hash, on the
  seeded 16-bit texts;
* the streaming tracker (pwm_gb300/csrc/host_stream.hpp) reports every word
  of a level exactly once, and only once all its bits are written;
* the host threads that fill and drain the pinned staging pieces
  (pwm_gb300/csrc/staging.hpp) copy exactly the bytes asked for."""
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
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-pthread", "-o", exe, SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def text_counts(text):
    t = np.asarray(text)
    nsym = 1 << (8 * t.dtype.itemsize)
    count = np.bincount(t.astype(np.int64), minlength=nsym)
    first = np.full(nsym, (1 << 64) - 1, dtype=np.uint64)
    syms, idx = np.unique(t, return_index=True)
    first[syms.astype(np.int64)] = idx
    return count, first


def codes(harness, text, tree, scale=1):
    t = np.asarray(text)
    count, first = text_counts(t)
    return codes_from_counts(harness, [int(c) * scale for c in count], first, t.dtype.itemsize, tree)


def codes_from_counts(harness, count, first, width, tree):
    inp = "%d\n" % len(count) + "".join("%d %d\n" % (int(c), int(f)) for c, f in zip(count, first))
    r = subprocess.run([harness, "huff", str(int(tree)), str(width)], input=inp, capture_output=True,
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


@pytest.mark.parametrize("tree", [False, True])
def test_code_tables_tie_heavy(harness, orc, tree):
    """2^16 symbols of 1..6 occurrences each: most counts, and most merged
    sums, tie, so the tables depend on the exact heap order of pwm's
    priority queue.  The builder's one-word heap items must give the oracle's
    tables, and counts scaled by 2^40 (too large for one-word items: the
    wide-item heap, the same comparisons) the same code lengths and words."""
    rng = np.random.default_rng(11)
    count = rng.integers(1, 7, size=1 << 16)
    text = np.repeat(np.arange(1 << 16, dtype=np.uint16), count)
    rng.shuffle(text)
    levels, sizes, ln, wd = codes(harness, text, tree)
    o_ln, o_wd, o_sizes, o_levels = orc.huff_codes(text, tree)
    assert levels == o_levels and sizes == [int(x) for x in o_sizes]
    assert ln == [int(x) for x in o_ln] and wd == [int(x) for x in o_wd]
    levels2, _, ln2, wd2 = codes(harness, text, tree, scale=1 << 40)
    assert levels2 == levels and ln2 == ln and wd2 == wd


def test_stream_tracker(harness):
    r = subprocess.run([harness, "lc", "2024", "3000"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def rev(x, bits):
    return int(format(x, "0%db" % bits)[::-1], 2) if bits else 0


def expected_plan(hist, L, tree, kmax, T):
    """The pass plan restated from first principles: a run of the matrix's
    level m starts at the count of elements whose key_m (first m bits, first
    bit least significant) is smaller, a run of the tree's at the count of
    elements with a smaller m-bit prefix."""
    n = int(hist.sum())
    cnt = {m: hist.reshape(1 << m, -1).sum(axis=1).astype(np.int64) for m in range(L + 1)}
    pn = {m: np.concatenate([[0], np.cumsum(cnt[m])]) for m in cnt}
    pk = {m: np.concatenate([[0], np.cumsum([cnt[m][rev(x, m)] for x in range(1 << m)])]) for m in cnt}
    zeros = [int(cnt[m + 1][0::2].sum()) for m in range(L)]
    regroup, passes, l = [], [], 0
    while l < L:
        K = min(kmax, L - l)
        out = l + K < L
        groups = 1 << l
        seg = tree and (l == 0 or (groups <= 65536 and n >= groups * 4 * T))
        TS = 2 * ((1 << K) - 1) + (1 << K)
        segs, tiles = [], 0
        if seg:
            for g in range(groups):
                m = int(cnt[l][rev(g, l)])
                if m == 0:
                    continue
                tab = [0] * TS
                for j in range(K):
                    for v in range(1 << j):
                        x = (v << l) | g
                        tab[(1 << j) - 1 + v] = int(pk[l + j][x])
                        tab[(1 << K) - 1 + (1 << j) - 1 + v] = int(pn[l + j][rev(x, l + j)])
                if out:
                    for v in range(1 << K):
                        tab[2 * ((1 << K) - 1) + v] = int(pk[l + K][(v << l) | g])
                segs.append((int(pk[l][g]), m, tiles, g, tab))
                tiles += (m + T - 1) // T
        else:
            tab = [0] * TS
            for j in range(K + (1 if out else 0)):
                ck = np.zeros(1 << j, dtype=np.int64)  # key of bits l..l+j-1, first least significant
                for p, c in enumerate(cnt[l + j]):
                    ck[rev(p & ((1 << j) - 1), j)] += c
                run = np.concatenate([[0], np.cumsum(ck)])[:-1]
                base = (1 << j) - 1 if j < K else 2 * ((1 << K) - 1)
                for v in range(1 << j):
                    tab[base + v] = int(run[v])
            segs.append((0, n, 0, 0, tab))
            tiles = (n + T - 1) // T
            if tree:
                regroup += [l + j for j in range(K) if l + j > 0]
        passes.append(((l, K, int(out), int(seg), tiles), segs))
        l += K
    return zeros, regroup, passes


def run_plan(harness, hist, L, tree, kmax, T):
    r = subprocess.run([harness, "plan", str(L), str(int(tree)), str(kmax), str(T)],
                       input=" ".join(str(int(x)) for x in hist), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().split("\n")
    zeros = [int(x) for x in lines[0].split()[1:]]
    regroup = [int(x) for x in lines[1].split()[1:]]
    passes, i = [], 2
    while i < len(lines):
        f = lines[i].split()
        head = tuple(int(x) for x in f[1:6])
        nseg = int(f[6])
        segs = []
        for s in range(nseg):
            a = [int(x) for x in lines[i + 1 + 2 * s].split()[1:]]
            tab = [int(x) for x in lines[i + 2 + 2 * s].split()[1:]]
            segs.append((a[0], a[1], a[2], a[3], tab))
        passes.append((head, segs))
        i += 1 + 2 * nseg
    return zeros, regroup, passes


@pytest.mark.parametrize("L,tree,kmax,T,scale", [
    (8, True, 4, 16384, 20000),   # both passes segmented (prefixes per group)
    (8, True, 4, 16384, 3),       # a small text: the second pass leaves the tree to the regroup
    (12, False, 4, 4096, 50),     # matrix only: one segment per pass
    (13, True, 3, 8192, 400),     # passes of 3 levels, segmented and not
    (6, True, 6, 16384, 9),       # all levels in one pass
    (1, True, 4, 16384, 7),
])
def test_pass_plan(harness, L, tree, kmax, T, scale):
    rng = np.random.default_rng(L * 7 + scale)
    hist = rng.integers(0, scale + 1, 1 << L).astype(np.int64)
    hist[rng.random(1 << L) < 0.2] = 0  # empty groups
    if hist.sum() == 0:
        hist[0] = 1
    assert run_plan(harness, hist, L, tree, kmax, T) == expected_plan(hist, L, tree, kmax, T)


def expected_merge(hists, L, tree):
    """pwm's merge order restated: level l of the merged structure is, block by
    block in the level's order (natural prefixes for the tree, bit-reversed
    for the matrix), the concatenation of the shards' runs of that block."""
    levels = []
    for l in range(L):
        counts = [h.reshape(1 << l, -1).sum(axis=1) for h in hists]
        runs, dst, rd = [], 0, [0] * len(hists)
        for b in range(1 << l):
            pfx = b if tree else rev(b, l)
            for s, c in enumerate(counts):
                if c[pfx]:
                    runs.append((dst, s, rd[s], int(c[pfx])))
                    dst += int(c[pfx])
                    rd[s] += int(c[pfx])
        assert dst == sum(int(h.sum()) for h in hists)
        levels.append(runs)
    return levels


@pytest.mark.parametrize("L,shards,tree", [(8, 4, True), (8, 4, False), (5, 7, True), (11, 3, False), (1, 2, True)])
def test_merge_plan(harness, L, shards, tree):
    rng = np.random.default_rng(L * 31 + shards)
    hists = [rng.integers(0, 20, 1 << L) * (rng.random(1 << L) < 0.6) for _ in range(shards)]
    hists[1 % shards][:] = 0  # an empty shard
    r = subprocess.run([harness, "merge", str(L), str(shards), str(int(tree))],
                       input=" ".join(str(int(x)) for h in hists for x in h), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got, cur = [], None
    for ln in r.stdout.strip().split("\n"):
        if ln.startswith("level"):
            cur = []
            got.append(cur)
        else:
            cur.append(tuple(int(x) for x in ln.split()))
    assert got == expected_merge(hists, L, tree)


def test_staging_copy_pool(harness):
    r = subprocess.run([harness, "copy", "7"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


@pytest.mark.parametrize("L,kmax,T,scale", [(9, 4, 4096, 50), (12, 4, 8192, 7), (16, 4, 16384, 3), (20, 4, 4096, 2),
                                           (13, 3, 4096, 9), (10, 1, 16384, 30), (11, 2, 4096, 0)])
def test_matrix_plan_from_digit_counts(harness, L, kmax, T, scale):
    """Deep matrix-only builds plan from the digit counts of each pass (what
    the device counts instead of a leaf histogram): same passes, tables and
    zero counts as the plan from every level's prefix counts."""
    rng = np.random.default_rng(L * 13 + kmax)
    hist = rng.integers(0, scale + 1, 1 << L).astype(np.int64)
    hist[rng.random(1 << L) < 0.3] = 0
    if hist.sum() == 0:
        hist[rng.integers(0, 1 << L)] = 5
    inp = "".join("%d\n" % int(h) for h in hist)
    r = subprocess.run([harness, "digits", str(L), str(kmax), str(T)], input=inp, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
