"""TEST INFRASTRUCTURE ONLY: ctypes wrappers for the oracle (liborc.so, the CPU
restatement of pwm's algorithms) and, where it was built, the reference shim
(_ref/libpwmref.so, pwm's own headers).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  The GPU product (pwm_gb300) never does.

All structures use the flat layout shared with the GPU library: every level
padded to a multiple of 16 u64 words (pwm's 128-byte cache-line alignment,
include/arrays/flat_two_dim_array.hpp:117-156).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_PATH = os.path.join(HERE, "liborc.so")
REF_PATH = os.path.join(HERE, "_ref", "libpwmref.so")

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_vp = ctypes.c_void_p

DTYPES = {1: np.uint8, 2: np.uint16, 4: np.uint32}


def reference_tree():
    """The pwm source tree named by the PWM_REFERENCE environment variable,
    or None when it is unset or absent."""
    p = os.environ.get("PWM_REFERENCE")
    return p if p and os.path.isdir(p) else None


def build(ref=False):
    """Compile liborc.so (and the reference shim when `ref` and the pwm
    source tree named by PWM_REFERENCE exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "liborc.so"], check=True)
    tree = reference_tree()
    if ref and tree:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={tree}"], check=True)


def _p(a, t=_u64p):
    return a.ctypes.data_as(t)


def padded_words(bits):
    return ((bits + 63) // 64 + 15) & ~15


def layout(level_bits):
    offs, off = [], 0
    for b in level_bits:
        offs.append(off)
        off += padded_words(int(b))
    return np.array(offs, dtype=np.uint64), off


class Structure:
    """A wavelet structure in the flat layout (host numpy arrays)."""

    def __init__(self, levels, level_bits, words, zeros, is_tree):
        self.levels = int(levels)
        self.level_bits = [int(b) for b in level_bits]
        self.offsets, self.total = layout(self.level_bits)
        self.words = words
        self.zeros = zeros
        self.is_tree = bool(is_tree)

    def level(self, l):
        o = int(self.offsets[l])
        return self.words[o:o + (self.level_bits[l] + 63) // 64]

    def same_bits(self, other):
        """Level-by-level equality of the meaningful words."""
        if self.levels != other.levels or self.level_bits != other.level_bits:
            return False
        return all(np.array_equal(self.level(l), other.level(l)) for l in range(self.levels))


class Oracle:
    def __init__(self, path=ORC_PATH):
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        self.L = L
        for name in ("orc_wx_ps", "orc_wx_pc", "orc_wx_naive"):
            f = getattr(L, name)
            f.argtypes = [_vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, _u64p, _u64p, _u64p]
            f.restype = ctypes.c_int
        for name in ("orc_wx_ppc", "orc_wx_dd_ps"):
            getattr(L, name).argtypes = [_vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                         _u64p, _u64p, _u64p, ctypes.c_int]
        L.orc_generate.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                   _vp, ctypes.c_int]
        L.orc_generate_batch.argtypes = [ctypes.c_uint64, ctypes.c_uint32, _u64p, _u32p, _vp]
        L.orc_rank_l0_size.argtypes = [ctypes.c_uint64]
        L.orc_rank_l0_size.restype = ctypes.c_uint64
        L.orc_rank_l12_size.argtypes = [ctypes.c_uint64]
        L.orc_rank_l12_size.restype = ctypes.c_uint64
        L.orc_rank_build.argtypes = [_u64p, ctypes.c_uint64, _u64p, _u32p]
        L.orc_select_build.argtypes = [ctypes.c_int, _u64p, ctypes.c_uint64, _u32p, _u32p]
        L.orc_select_build.restype = ctypes.c_uint64
        L.orc_select.argtypes = [ctypes.c_int, _u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64, _u32p, _u32p,
                                 ctypes.c_uint64, ctypes.c_uint64]
        L.orc_select.restype = ctypes.c_uint64
        L.orc_rank1.argtypes = [_u64p, ctypes.c_uint64, _u64p, _u32p, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_total_ones.argtypes = [_u64p, ctypes.c_uint64, _u32p]
        L.orc_total_ones.restype = ctypes.c_uint64
        L.orc_rank1.restype = ctypes.c_uint64
        L.orc_word_select1.argtypes = [ctypes.c_uint64, ctypes.c_uint32]
        L.orc_word_select1.restype = ctypes.c_uint32
        L.orc_qs_create.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_uint64, _u64p, _u64p, _u64p]
        L.orc_qs_create.restype = _vp
        L.orc_qs_free.argtypes = [_vp]
        L.orc_qs_blocks.argtypes = [_vp, ctypes.c_uint32, _u64p, _u32p, _u32p, _u32p, _u64p]
        for name in ("orc_qs_access",):
            getattr(L, name).argtypes = [_vp, ctypes.c_uint64]
            getattr(L, name).restype = ctypes.c_uint64
        for name in ("orc_qs_rank", "orc_qs_select"):
            getattr(L, name).argtypes = [_vp, ctypes.c_uint64, ctypes.c_uint64]
            getattr(L, name).restype = ctypes.c_uint64
        L.orc_cpu_step.argtypes = [_vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, _u64p,
                                   _u64p, _u64p, _u64p, ctypes.c_int]
        L.orc_huff_codes.argtypes = [_vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, _u64p, _u64p,
                                     ctypes.c_uint64, _u64p, _u32p]
        L.orc_huff_codes.restype = ctypes.c_uint64
        L.orc_huff_naive.argtypes = [_vp, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, _u64p, _u64p,
                                     ctypes.c_uint32, _u64p, _u64p, _u64p]
        L.orc_copy_bits_u8.argtypes = [_vp, _vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_copy_bits_u64.argtypes = [_vp, _vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]

    @staticmethod
    def reduce_alphabet(text):
        """pwm's reduce_alphabet (include/util/alphabet_util.hpp:18-45): the
        symbols renumbered 0, 1, ... in order of first occurrence; returns
        (renumbered text, distinct symbols - 1), the latter all ones (0 - 1
        in uint64) for an empty text.  Pinned by tests/golden/alphabet.json,
        outputs of pwm's own function."""
        t = np.asarray(text)
        if t.size == 0:
            return t.copy(), (1 << 64) - 1
        syms, first = np.unique(t, return_index=True)
        rank = np.empty(syms.size, dtype=np.uint64)
        rank[np.argsort(first, kind="stable")] = np.arange(syms.size, dtype=np.uint64)
        return rank[np.searchsorted(syms, t)].astype(t.dtype), syms.size - 1

    def copy_bits(self, dst, src, dst_off, src_off, length):
        """pwm's copy_bits (merge.hpp:19-190) on numpy arrays of uint8 or
        uint64 words; dst is updated in place."""
        f = self.L.orc_copy_bits_u8 if dst.dtype == np.uint8 else self.L.orc_copy_bits_u64
        f(dst.ctypes.data, src.ctypes.data, int(dst_off), int(src_off), int(length))

    # -- construction ------------------------------------------------------
    def build(self, text, levels, is_tree, variant="ps", threads=0):
        text = np.ascontiguousarray(text)
        n, w = text.size, text.dtype.itemsize
        bits = [n] * levels
        offs, total = layout(bits)
        words = np.zeros(max(total, 1), dtype=np.uint64)
        zeros = np.zeros(max(levels, 1), dtype=np.uint64)
        f = {"ps": self.L.orc_wx_ps, "pc": self.L.orc_wx_pc, "naive": self.L.orc_wx_naive,
             "ppc": self.L.orc_wx_ppc, "dd_ps": self.L.orc_wx_dd_ps}[variant]
        args = [text.ctypes.data_as(_vp), n, w, levels, int(is_tree), _p(words), _p(offs), _p(zeros)]
        if variant in ("ppc", "dd_ps"):
            args.append(threads)
        f(*args)
        if n == 0:
            return Structure(0, [], words[:0], zeros[:0], is_tree)
        return Structure(levels, bits, words, None if is_tree else zeros[:levels], is_tree)

    def cpu_step_buffers(self, n, levels):
        offs, total = layout([n] * levels)
        return (np.zeros(max(total, 1), dtype=np.uint64), np.zeros(max(total, 1), dtype=np.uint64), offs,
                np.zeros(max(levels, 1), dtype=np.uint64))

    CPU_VARIANTS = {"ppc": 0, "dd_ps": 1}

    def cpu_step(self, text, levels, threads, bufs, variant="ppc"):
        """CPU baseline step: matrix + tree with pwm's parallel prefix
        counting (wx_ppc) or domain decomposition (wx_dd_ps), then
        rank/select support of every level."""
        wm, wt, offs, zeros = bufs
        self.L.orc_cpu_step(text.ctypes.data_as(_vp), text.size, text.dtype.itemsize, levels, threads, _p(wm), _p(wt),
                            _p(offs), _p(zeros), self.CPU_VARIANTS[variant])

    def generate(self, dist, seed, n, width, param=0, threads=0):
        """Seeded synthetic text, identical to pwm_gb300.generate (the shared
        generator header), produced without the GPU library."""
        out = np.empty(n, dtype=DTYPES[width])
        if n:
            self.L.orc_generate(int(dist), int(seed), int(param), int(n), int(width), out.ctypes.data_as(_vp),
                                int(threads))
        return out

    def generate_batch(self, seed, count):
        """The batched workload's texts (pwm_gb300.generate_batch's)."""
        offs = np.zeros(count + 1, dtype=np.uint64)
        levels = np.zeros(max(count, 1), dtype=np.uint32)
        self.L.orc_generate_batch(int(seed), int(count), _p(offs), _p(levels, _u32p), None)
        texts = np.zeros(max(int(offs[-1]), 1), dtype=np.uint8)
        self.L.orc_generate_batch(int(seed), int(count), _p(offs), _p(levels, _u32p), texts.ctypes.data_as(_vp))
        return texts[:int(offs[-1])], offs, levels[:count]

    # -- rank / select -----------------------------------------------------
    def rank_select_blocks(self, level_words):
        lw = np.ascontiguousarray(level_words, dtype=np.uint64)
        nw = lw.size
        n0 = self.L.orc_rank_l0_size(nw)
        n12 = self.L.orc_rank_l12_size(nw)
        l0 = np.zeros(n0, dtype=np.uint64)
        l12 = np.zeros(2 * n12, dtype=np.uint32)
        buf = lw if nw else np.zeros(1, dtype=np.uint64)
        self.L.orc_rank_build(_p(buf), nw, _p(l0), _p(l12, _u32p))
        cap = nw * 64 // 8192 + 2
        s0 = np.zeros(cap, dtype=np.uint32)
        s1 = np.zeros(cap, dtype=np.uint32)
        ns0 = self.L.orc_select_build(0, _p(buf), nw, _p(l12, _u32p), _p(s0, _u32p))
        ns1 = self.L.orc_select_build(1, _p(buf), nw, _p(l12, _u32p), _p(s1, _u32p))
        return l0, l12, s0[:ns0], s1[:ns1]

    def select(self, value, level_words, occ, blocks=None):
        lw = np.ascontiguousarray(level_words, dtype=np.uint64)
        l0, l12, s0, s1 = blocks if blocks is not None else self.rank_select_blocks(lw)
        smp = s1 if value else s0
        smp_buf = smp if smp.size else np.zeros(1, dtype=np.uint32)
        buf = lw if lw.size else np.zeros(1, dtype=np.uint64)
        return np.array([self.L.orc_select(value, _p(buf), lw.size, _p(l0), l0.size, _p(l12, _u32p),
                                           _p(smp_buf, _u32p), smp.size, int(o)) for o in occ], dtype=np.uint64)

    def rank1(self, level_words, idx, blocks=None):
        lw = np.ascontiguousarray(level_words, dtype=np.uint64)
        l0, l12, _, _ = blocks if blocks is not None else self.rank_select_blocks(lw)
        buf = lw if lw.size else np.zeros(1, dtype=np.uint64)
        ones = self.L.orc_total_ones(_p(buf), lw.size, _p(l12, _u32p))
        return np.array([self.L.orc_rank1(_p(buf), lw.size, _p(l0), _p(l12, _u32p), ones, int(i)) for i in idx],
                        dtype=np.uint64)

    def query_support(self, s):
        return OracleQueries(self, s)

    # -- Huffman -----------------------------------------------------------
    def huff_codes(self, text, is_tree):
        text = np.ascontiguousarray(text)
        n, w = text.size, text.dtype.itemsize
        cap = 1 << (8 * w) if w < 4 else int(text.max()) + 1 if n else 1
        ln = np.zeros(cap, dtype=np.uint64)
        wd = np.zeros(cap, dtype=np.uint64)
        sizes = np.zeros(64, dtype=np.uint64)
        lv = ctypes.c_uint32(0)
        nsym = self.L.orc_huff_codes(text.ctypes.data_as(_vp), n, w, int(is_tree), _p(ln), _p(wd), cap,
                                     _p(sizes), ctypes.byref(lv))
        return ln[:nsym].copy(), wd[:nsym].copy(), sizes[:lv.value].copy(), lv.value

    def huff_build(self, text, is_tree, codes=None):
        text = np.ascontiguousarray(text)
        n, w = text.size, text.dtype.itemsize
        if codes is None:
            codes = self.huff_codes(text, is_tree)
        ln, wd, sizes, levels = codes
        offs, total = layout(sizes)
        words = np.zeros(max(total, 1), dtype=np.uint64)
        zeros = np.zeros(max(levels, 1), dtype=np.uint64)
        if n:
            self.L.orc_huff_naive(text.ctypes.data_as(_vp), n, w, int(is_tree), _p(ln), _p(wd), levels,
                                  _p(words), _p(offs), _p(zeros))
        return Structure(levels, list(sizes), words, None if is_tree else zeros[:levels], is_tree)


class OracleQueries:
    def __init__(self, orc, s):
        self.orc, self.s = orc, s
        z = s.zeros if s.zeros is not None else np.zeros(max(s.levels, 1), dtype=np.uint64)
        self._z = np.ascontiguousarray(z, dtype=np.uint64)
        n = s.level_bits[0] if s.levels else 0
        self.h = orc.L.orc_qs_create(s.levels, int(s.is_tree), n, _p(s.words), _p(s.offsets), _p(self._z))

    def __del__(self):
        if getattr(self, "h", None):
            self.orc.L.orc_qs_free(self.h)
            self.h = None

    def access(self, i):
        return self.orc.L.orc_qs_access(self.h, i)

    def rank(self, sym, i):
        return self.orc.L.orc_qs_rank(self.h, sym, i)

    def select(self, sym, occ):
        return self.orc.L.orc_qs_select(self.h, sym, occ)

    def blocks(self, level):
        counts = np.zeros(4, dtype=np.uint64)
        self.orc.L.orc_qs_blocks(self.h, level, None, None, None, None, _p(counts))
        n0, n12, ns0, ns1 = (int(c) for c in counts)
        l0 = np.zeros(max(n0, 1), dtype=np.uint64)
        l12 = np.zeros(max(2 * n12, 1), dtype=np.uint32)
        s0 = np.zeros(max(ns0, 1), dtype=np.uint32)
        s1 = np.zeros(max(ns1, 1), dtype=np.uint32)
        self.orc.L.orc_qs_blocks(self.h, level, _p(l0), _p(l12, _u32p), _p(s0, _u32p), _p(s1, _u32p), _p(counts))
        return l0[:n0], l12[:2 * n12], s0[:ns0], s1[:ns1]


class Reference:
    """pwm's own code (only where oracle/_ref/libpwmref.so was built)."""

    VARIANTS = {"ps": 0, "pc": 1, "naive": 2, "ppc": 3, "pps": 4, "dd_ps": 5, "dd_pc": 6, "pc_ss": 7,
                "ppc_ss": 8, "dd_pc_ss": 9}
    HUFF = {"naive": 0, "ps": 1, "pc": 2}

    @staticmethod
    def available():
        return os.path.exists(REF_PATH)

    def __init__(self):
        L = ctypes.CDLL(REF_PATH)
        self.L = L
        L.pwmref_fixture_count.restype = ctypes.c_uint64
        L.pwmref_fixture.argtypes = [ctypes.c_uint64, ctypes.c_char_p, ctypes.c_uint64]
        L.pwmref_fixture.restype = ctypes.c_uint64
        L.pwmref_build.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_int, _vp, ctypes.c_uint64, ctypes.c_uint64,
                                   _u64p, ctypes.c_uint64, _u64p, _u64p, _u32p]
        L.pwmref_build.restype = ctypes.c_uint64
        L.pwmref_huff.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_int, _vp, ctypes.c_uint64, _u64p,
                                  ctypes.c_uint64, _u64p, _u64p, _u32p, _u64p, _u64p, ctypes.c_uint64, _u64p]
        L.pwmref_huff.restype = ctypes.c_uint64
        L.pwmref_rank_select.argtypes = [_u64p, ctypes.c_uint64, _u64p, _u32p, _u32p, _u32p, _u64p]
        L.pwmref_rank1.argtypes = [_u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64, _u64p]
        L.pwmref_select.argtypes = [ctypes.c_int, _u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64, _u64p]
        L.pwmref_queries.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                     _u64p, _u64p, ctypes.c_uint64, _u64p]
        L.pwmref_copy_bits_u8.argtypes = [_vp, _vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.pwmref_copy_bits_u64.argtypes = [_vp, _vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.pwmref_reduce_alphabet.argtypes = [ctypes.c_uint32, _vp, ctypes.c_uint64]
        L.pwmref_reduce_alphabet.restype = ctypes.c_uint64

    def reduce_alphabet(self, text):
        """pwm's own reduce_alphabet: (renumbered copy, max_char)."""
        t = np.ascontiguousarray(text).copy()
        m = self.L.pwmref_reduce_alphabet(t.dtype.itemsize, t.ctypes.data_as(_vp), t.size)
        return t, m

    def copy_bits(self, dst, src, dst_off, src_off, length):
        """pwm's copy_bits on numpy arrays of uint8 or uint64 words (dst in place)."""
        f = self.L.pwmref_copy_bits_u8 if dst.dtype == np.uint8 else self.L.pwmref_copy_bits_u64
        f(dst.ctypes.data, src.ctypes.data, int(dst_off), int(src_off), int(length))

    def fixtures(self):
        out = []
        for i in range(self.L.pwmref_fixture_count()):
            n = self.L.pwmref_fixture(i, None, 0)
            buf = ctypes.create_string_buffer(max(n, 1))
            self.L.pwmref_fixture(i, buf, n)
            out.append(np.frombuffer(buf.raw[:n], dtype=np.uint8).copy())
        return out

    def build(self, text, levels, is_tree, variant="ps"):
        text = np.ascontiguousarray(text)
        n, w = text.size, text.dtype.itemsize
        offs, total = layout([n] * levels)
        words = np.zeros(max(total, 1), dtype=np.uint64)
        bits = np.zeros(max(levels, 1), dtype=np.uint64)
        zeros = np.zeros(max(levels, 1), dtype=np.uint64)
        lv = ctypes.c_uint32(0)
        self.L.pwmref_build(self.VARIANTS[variant], w, int(is_tree), text.ctypes.data_as(_vp), n, levels,
                            _p(words), total, _p(bits), _p(zeros), ctypes.byref(lv))
        lv = lv.value
        return Structure(lv, list(bits[:lv]), words, None if is_tree else zeros[:lv], is_tree)

    def huff(self, text, is_tree, variant="naive"):
        text = np.ascontiguousarray(text)
        n, w = text.size, text.dtype.itemsize
        cap_codes = 1 << 20 if w == 4 else 1 << (8 * w)
        ln = np.zeros(cap_codes, dtype=np.uint64)
        wd = np.zeros(cap_codes, dtype=np.uint64)
        nc = ctypes.c_uint64(0)
        lv = ctypes.c_uint32(0)
        bits = np.zeros(64, dtype=np.uint64)
        zeros = np.zeros(64, dtype=np.uint64)
        total = self.L.pwmref_huff(self.HUFF[variant], w, int(is_tree), text.ctypes.data_as(_vp), n, None, 0,
                                   _p(bits), None, ctypes.byref(lv), _p(ln), _p(wd), cap_codes, ctypes.byref(nc))
        words = np.zeros(max(total, 1), dtype=np.uint64)
        self.L.pwmref_huff(self.HUFF[variant], w, int(is_tree), text.ctypes.data_as(_vp), n, _p(words), total,
                           _p(bits), _p(zeros), ctypes.byref(lv), _p(ln), _p(wd), cap_codes, ctypes.byref(nc))
        lv = lv.value
        s = Structure(lv, list(bits[:lv]), words, None if is_tree else zeros[:lv], is_tree)
        return s, (ln[:nc.value].copy(), wd[:nc.value].copy())

    def rank_select_blocks(self, level_words):
        lw = np.ascontiguousarray(level_words, dtype=np.uint64)
        buf = lw if lw.size else np.zeros(1, dtype=np.uint64)
        counts = np.zeros(4, dtype=np.uint64)
        self.L.pwmref_rank_select(_p(buf), lw.size, None, None, None, None, _p(counts))
        n0, n12, ns0, ns1 = (int(c) for c in counts)
        l0 = np.zeros(max(n0, 1), dtype=np.uint64)
        l12 = np.zeros(max(2 * n12, 1), dtype=np.uint32)
        s0 = np.zeros(max(ns0, 1), dtype=np.uint32)
        s1 = np.zeros(max(ns1, 1), dtype=np.uint32)
        self.L.pwmref_rank_select(_p(buf), lw.size, _p(l0), _p(l12, _u32p), _p(s0, _u32p), _p(s1, _u32p), _p(counts))
        return l0[:n0], l12[:2 * n12], s0[:ns0], s1[:ns1]

    def select(self, value, level_words, occ):
        lw = np.ascontiguousarray(level_words, dtype=np.uint64)
        occ = np.ascontiguousarray(occ, dtype=np.uint64)
        out = np.zeros(occ.size, dtype=np.uint64)
        self.L.pwmref_select(value, _p(lw), lw.size, _p(occ), occ.size, _p(out))
        return out

    def queries(self, is_tree, text, levels, op, a, b=None):
        text = np.ascontiguousarray(text, dtype=np.uint8)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b if b is not None else np.zeros_like(a), dtype=np.uint64)
        out = np.zeros(a.size, dtype=np.uint64)
        self.L.pwmref_queries(int(is_tree), text.tobytes(), text.size, levels, op, _p(a), _p(b), a.size, _p(out))
        return out
