"""pwm_gb300: GB300-native wavelet tree / wavelet matrix construction.

A host-side mirror of kurpicz/pwm's construction API over the C ABI of
libpwmgpu.so (include/pwmgpu.h):

* ``wx_ps``, ``wx_pc``, ``wx_ppc``, ``wx_pps``, ``wx_pc_ss``, ``wx_ppc_ss``,
  ``wx_dd_ps``, ``wx_dd_pc``, ``wx_dd_pc_ss`` (pwm include/wx_*.hpp) and the
  Huffman-shaped ``wx_huff_ps``, ``wx_huff_pc``, ``wx_huff_pc_ss``,
  ``wx_huff_naive`` (include/wx_huff_*.hpp): construction classes whose
  ``compute(text, size, levels)`` returns a ``wavelet_structure``.  All of a
  plain kind produce pwm's identical bit vectors, so they share one GPU path.
* ``wavelet_structure`` (include/construction/wavelet_structure.hpp:142-199)
  with ``levels()``, ``bvs()``, ``zeros()``, ``is_tree()``,
  ``is_huffman_shaped()``, ``text_size()``.
* ``algorithm_list`` / ``CONSTRUCTION_REGISTER``
  (include/benchmark/algorithm.hpp:39-81, 273-279): the registry.
* ``DeviceStructure``: a device-resident build with rank/select support and
  batched access/rank/select queries (include/queries/query_support.hpp).

Every compute runs on the GPU; there is no CPU fallback.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import (GEN_DNA4, GEN_MIX16, GEN_UNIFORM, GEN_ZIPF256, KEEP_HISTOGRAM, MATRIX, Q_ACCESS, Q_RANK, Q_SELECT,
                   RANK_SELECT, TREE, PwmGpuError)

__all__ = ["Context", "default_context", "wavelet_structure", "bit_vectors", "algorithm_list",
           "CONSTRUCTION_REGISTER", "DeviceStructure", "Batch", "generate", "generate_batch", "huffman_codes",
           "PwmGpuError"]

_WIDTH_DTYPE = {1: np.uint8, 2: np.uint16, 4: np.uint32}


def _u64p(a):
    return a.ctypes.data_as(_lib.u64p)


def _u32p(a):
    return a.ctypes.data_as(_lib.u32p)


def padded_words(bits):
    return ((int(bits) + 63) // 64 + 15) & ~15


class Context:
    """A pwmgpu context: one device, one CUDA stream, cached scratch."""

    def __init__(self, device=0, stream=None):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        st = self.lib.pwmgpu_ctx_create(device, stream, ctypes.byref(h))
        if st != 0:
            raise PwmGpuError(st, "pwmgpu_ctx_create failed (is a GB300 visible?)")
        self.h = h
        self.device = device

    def check(self, st):
        if st != 0:
            msg = self.lib.pwmgpu_ctx_last_error(self.h)
            raise PwmGpuError(st, msg.decode() if msg else "")

    def sync(self):
        self.check(self.lib.pwmgpu_ctx_sync(self.h))

    @property
    def launches(self):
        return int(self.lib.pwmgpu_ctx_launch_count(self.h))

    def set_pass_levels(self, k):
        self.check(self.lib.pwmgpu_ctx_set_pass_levels(self.h, int(k)))

    def set_engine(self, engine):
        """ENGINE_TILE (default) or ENGINE_WARP for plain builds."""
        self.check(self.lib.pwmgpu_ctx_set_engine(self.h, int(engine)))

    def set_upload_piece_bytes(self, nbytes):
        """Piece size of pinned host-text uploads (default 64 MiB)."""
        self.check(self.lib.pwmgpu_ctx_set_upload_piece_bytes(self.h, int(nbytes)))

    def set_host_copy_threads(self, threads):
        """Host threads that move pageable buffers through pinned staging
        pieces (-1: automatic, up to 8; 0: unstaged driver copies)."""
        self.check(self.lib.pwmgpu_ctx_set_host_copy_threads(self.h, int(threads)))

    def release_scratch(self):
        """Frees the buffers and cached structures the context keeps between calls."""
        self.check(self.lib.pwmgpu_ctx_release_scratch(self.h))

    def set_stream_chunks(self, chunks):
        """Chunks of the passes whose words stream to pinned outputs (1..16, default 4)."""
        self.check(self.lib.pwmgpu_ctx_set_stream_chunks(self.h, int(chunks)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.pwmgpu_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


ENGINE_TILE = 0
ENGINE_WARP = 1

_default = None


def default_context():
    global _default
    if _default is None:
        _default = Context()
    return _default


class bit_vectors:
    """pwm's bit_vectors (include/arrays/bit_vectors.hpp:13-29): levels in one
    allocation, each padded to 128 bytes."""

    def __init__(self, level_bits, words=None):
        self.level_bits_ = [int(b) for b in level_bits]
        offs, off = [], 0
        for b in self.level_bits_:
            offs.append(off)
            off += padded_words(b)
        self.offsets = offs
        self.total_words = off
        self.data = np.zeros(max(off, 1), dtype=np.uint64) if words is None else words

    def levels(self):
        return len(self.level_bits_)

    def level_bit_size(self, level):
        return self.level_bits_[level]

    def __getitem__(self, level):
        o = self.offsets[level]
        return self.data[o:o + (self.level_bits_[level] + 63) // 64]


class wavelet_structure:
    """pwm's wavelet_structure (include/construction/wavelet_structure.hpp)."""

    def __init__(self, bvs, zeros, is_tree, is_huffman_shaped=False, codes=None):
        self._bvs = bvs
        self._zeros = list(zeros) if zeros is not None else []
        self._is_tree = bool(is_tree)
        self._huff = bool(is_huffman_shaped)
        self._codes = codes

    def levels(self):
        return self._bvs.levels()

    def bvs(self):
        return self._bvs

    def zeros(self):
        return self._zeros

    def is_tree(self):
        return self._is_tree

    def is_huffman_shaped(self):
        return self._huff

    def text_size(self):
        return self._bvs.level_bit_size(0) if self._bvs.levels() else 0

    def codes(self):
        return self._codes


def _as_text(text, size, word_width):
    a = np.ascontiguousarray(text)
    if a.dtype != _WIDTH_DTYPE[word_width]:
        a = a.astype(_WIDTH_DTYPE[word_width])
    if size > a.size:
        raise ValueError("size exceeds the text")
    return a[:size]


class _PlainConstruction:
    """compute() of pwm's plain wx_* classes (include/wx_ps.hpp:37-56 and
    siblings) on the GPU."""

    is_huffman_shaped = False
    is_parallel = True
    external_in = False
    external_out = False
    stats_support = False
    is_inplace = False

    def __init__(self, alphabet=np.uint8, is_tree=False, context=None):
        self.alphabet = np.dtype(alphabet)
        self.word_width = self.alphabet.itemsize
        self.is_tree = bool(is_tree)
        self.ctx = context

    def compute(self, text, size, levels):
        ctx = self.ctx or default_context()
        size, levels = int(size), int(levels)
        if size == 0:
            return wavelet_structure(bit_vectors([]), [] if not self.is_tree else None, self.is_tree)
        t = _as_text(text, size, self.word_width)
        bvs = bit_vectors([size] * levels)
        zeros = np.zeros(levels, dtype=np.uint64)
        ctx.check(ctx.lib.pwmgpu_compute(ctx.h, t.ctypes.data, size, self.word_width, levels, int(self.is_tree),
                                         _u64p(bvs.data), _u64p(zeros)))
        return wavelet_structure(bvs, None if self.is_tree else [int(z) for z in zeros], self.is_tree)


class _HuffmanConstruction(_PlainConstruction):
    """compute() of pwm's Huffman-shaped wx_huff_* classes
    (include/wx_huff_ps.hpp:45-79 and siblings) on the GPU.  `levels` is
    ignored, as in pwm; codes come from pwm's canonical builder semantics
    (huffman_codes) or from `codes=(code_len, code_word)`."""

    is_huffman_shaped = True

    def compute(self, text, size, levels=0, codes=None):
        ctx = self.ctx or default_context()
        size = int(size)
        t = _as_text(text, size, self.word_width)
        if codes is None:
            codes = huffman_codes(t, self.is_tree, ctx)
        code_len = np.ascontiguousarray(codes[0], dtype=np.uint64)
        code_word = np.ascontiguousarray(codes[1], dtype=np.uint64)
        if size == 0:
            return wavelet_structure(bit_vectors([]), None if self.is_tree else [], self.is_tree, True, codes)
        if len(codes) >= 4:
            # huffman_codes() already returns the level sizes of this text
            L = int(codes[3])
            sizes = [int(x) for x in codes[2][:L]]
        else:
            # level sizes from the symbol counts (huff_level_sizes_builder.hpp:13-46): one pass over the text
            counts = np.bincount(t, minlength=code_len.size)[:code_len.size] if code_len.size else \
                np.zeros(0, dtype=np.int64)
            present = code_len[counts > 0]
            L = int(present.max()) if present.size else 0
            sizes = [int(counts[code_len > l].sum()) for l in range(L)] if L else []
        bvs = bit_vectors(sizes)
        zeros = np.zeros(max(L, 1), dtype=np.uint64)
        sz = np.array(sizes if sizes else [0], dtype=np.uint64)
        ctx.check(ctx.lib.pwmgpu_compute_huffman(ctx.h, t.ctypes.data, size, self.word_width, int(self.is_tree),
                                                 _u64p(code_len), _u64p(code_word), code_len.size, L, _u64p(sz),
                                                 _u64p(bvs.data), _u64p(zeros)))
        return wavelet_structure(bvs, None if self.is_tree else [int(z) for z in zeros[:L]], self.is_tree, True,
                                 (code_len, code_word))


def huffman_codes(text, is_tree, context=None):
    """pwm's canonical Huffman codes of an 8- or 16-bit text: (code_len,
    code_word, level_sizes, levels), with max_symbol+1 table entries."""
    ctx = context or default_context()
    t = np.ascontiguousarray(text)
    w = t.dtype.itemsize
    cap = 1 << (8 * w)
    ln = np.zeros(cap, dtype=np.uint64)
    wd = np.zeros(cap, dtype=np.uint64)
    nc = ctypes.c_uint64(0)
    lv = ctypes.c_uint32(0)
    sizes = np.zeros(64, dtype=np.uint64)
    ctx.check(ctx.lib.pwmgpu_huffman_codes(ctx.h, t.ctypes.data, t.size, w, int(is_tree), _u64p(ln), _u64p(wd), cap,
                                           ctypes.byref(nc), _u64p(sizes), ctypes.byref(lv)))
    return ln[:nc.value].copy(), wd[:nc.value].copy(), sizes[:lv.value].copy(), lv.value


def reduce_alphabet(d_text_ptr, size, word_width, d_out_ptr=None, context=None):
    """pwm's reduce_alphabet on a device text (pwmgpu_reduce_alphabet):
    symbols renumbered by first occurrence into d_out_ptr (default: in
    place); returns max_char = distinct symbols - 1."""
    ctx = context or default_context()
    mc = ctypes.c_uint64(0)
    out = d_text_ptr if d_out_ptr is None else d_out_ptr
    ctx.check(ctx.lib.pwmgpu_reduce_alphabet(ctx.h, ctypes.c_void_p(int(d_text_ptr)), int(size), int(word_width),
                                             ctypes.c_void_p(int(out)), ctypes.byref(mc)))
    return mc.value


def compute_semi_external(text, levels, matrix=True, tree=True, device_budget=0, context=None, out=None):
    """Semi-external build of a host text (pwmgpu_compute_semi_external):
    the text streams through the GPU in pieces within about device_budget
    bytes.  Returns (matrix words, matrix zeros, tree words) in the layout of
    DeviceStructure.download (None for a structure not asked for).  out:
    optional (matrix, tree) u64 arrays to fill (e.g. pinned memory)."""
    ctx = context or default_context()
    t = np.ascontiguousarray(text)
    n, w = t.size, t.dtype.itemsize
    lw = (((n + 63) // 64) + 15) // 16 * 16
    if out is None:
        out = (np.zeros(levels * lw, np.uint64) if matrix else None, np.zeros(levels * lw, np.uint64) if tree else None)
    wm, wt = out
    zeros = np.zeros(levels, np.uint64) if matrix else None
    cast = lambda a: _u64p(a) if isinstance(a, np.ndarray) else (
        ctypes.cast(ctypes.c_void_p(int(a.data_ptr())), _lib.u64p) if a is not None else None)
    ctx.check(ctx.lib.pwmgpu_compute_semi_external(ctx.h, ctypes.c_void_p(t.ctypes.data), n, w, int(levels), cast(wm),
                                                   _u64p(zeros) if zeros is not None else None, cast(wt),
                                                   int(device_budget)))
    return wm, zeros, wt


def _variant(name, base, doc):
    return type(name, (base,), {"__doc__": doc})


wx_ps = _variant("wx_ps", _PlainConstruction, "pwm include/wx_ps.hpp:19-57 (prefix sorting)")
wx_pc = _variant("wx_pc", _PlainConstruction, "pwm include/wx_pc.hpp:19-58 (prefix counting)")
wx_ppc = _variant("wx_ppc", _PlainConstruction, "pwm include/wx_ppc.hpp (parallel prefix counting)")
wx_pps = _variant("wx_pps", _PlainConstruction, "pwm include/wx_pps.hpp:21-70 (parallel prefix sorting)")
wx_pc_ss = _variant("wx_pc_ss", _PlainConstruction, "pwm include/wx_pc_ss.hpp (single scan)")
wx_ppc_ss = _variant("wx_ppc_ss", _PlainConstruction, "pwm include/wx_ppc_ss.hpp (parallel single scan)")
wx_dd_ps = _variant("wx_dd_ps", _PlainConstruction, "pwm include/wx_dd_ps.hpp:26-121 (domain decomposition)")
wx_dd_pc = _variant("wx_dd_pc", _PlainConstruction, "pwm include/wx_dd_pc.hpp:26-120")
wx_dd_pc_ss = _variant("wx_dd_pc_ss", _PlainConstruction, "pwm include/wx_dd_pc_ss.hpp:25-119")
wx_huff_ps = _variant("wx_huff_ps", _HuffmanConstruction, "pwm include/wx_huff_ps.hpp:24-80")
wx_huff_pc = _variant("wx_huff_pc", _HuffmanConstruction, "pwm include/wx_huff_pc.hpp:24-81")
wx_huff_pc_ss = _variant("wx_huff_pc_ss", _HuffmanConstruction, "pwm include/wx_huff_pc_ss.hpp:24-78")
wx_huff_naive = _variant("wx_huff_naive", _HuffmanConstruction, "pwm include/wx_huff_naive.hpp:24-80")

__all__ += ["wx_ps", "wx_pc", "wx_ppc", "wx_pps", "wx_pc_ss", "wx_ppc_ss", "wx_dd_ps", "wx_dd_pc", "wx_dd_pc_ss",
            "wx_huff_ps", "wx_huff_pc", "wx_huff_pc_ss", "wx_huff_naive"]


class construction_algorithm:
    """pwm's construction_algorithm (include/benchmark/algorithm.hpp:83-191)."""

    def __init__(self, name, description, impl):
        self._name, self._description, self.impl = name, description, impl

    def name(self):
        return self._name

    def description(self):
        return self._description

    def is_parallel(self):
        return self.impl.is_parallel

    def is_tree(self):
        return self.impl.is_tree

    def is_huffman_shaped(self):
        return self.impl.is_huffman_shaped

    def is_inplace(self):
        return self.impl.is_inplace

    def word_width(self):
        return self.impl.word_width

    def compute_bitvector(self, text, size, levels):
        return self.impl.compute(text, size, levels)

    compute_internal_bitvector = compute_bitvector

    def huffman_bit_size(self, text, size, levels):
        if not self.impl.is_huffman_shaped:
            return 0
        ws = self.impl.compute(text, size, levels)
        return sum(ws.bvs().level_bit_size(l) for l in range(ws.levels()))

    def print_info(self):
        print(f"{self._name}: {self._description}")


class algorithm_list:
    """pwm's algorithm_list<ext_in, ext_out, word_width> (algorithm.hpp:39-81),
    internal memory only."""

    _lists = {}

    @classmethod
    def get_algorithm_list(cls, word_width=1):
        return cls._lists.setdefault(int(word_width), [])

    @classmethod
    def register_algorithm(cls, algo):
        cls.get_algorithm_list(algo.word_width()).append(algo)

    @classmethod
    def filtered(cls, f, word_width=1):
        return [a for a in cls.get_algorithm_list(word_width) if f(a)]


def CONSTRUCTION_REGISTER(name, description, impl):
    """pwm's CONSTRUCTION_REGISTER (algorithm.hpp:273-279)."""
    algo = construction_algorithm(name, description, impl)
    algorithm_list.register_algorithm(algo)
    return algo


def _register_all():
    names = {"ps": wx_ps, "pc": wx_pc, "ppc": wx_ppc, "pps": wx_pps, "pc_ss": wx_pc_ss, "ppc_ss": wx_ppc_ss,
             "dd_ps": wx_dd_ps, "dd_pc": wx_dd_pc, "dd_pc_ss": wx_dd_pc_ss}
    for tree in (False, True):
        pre = "wt" if tree else "wm"
        for dt in (np.uint8, np.uint16, np.uint32):
            for key, cls in names.items():
                CONSTRUCTION_REGISTER(f"{pre}_gpu_{key}",
                                      f"GB300 {'wavelet tree' if tree else 'wavelet matrix'} construction with "
                                      f"{np.dtype(dt).itemsize * 8}-bit alphabet ({key} semantics).", cls(dt, tree))
            if dt != np.uint32:
                for key, cls in (("huff_ps", wx_huff_ps), ("huff_pc", wx_huff_pc), ("huff_naive", wx_huff_naive)):
                    CONSTRUCTION_REGISTER(f"{pre}_gpu_{key}", f"GB300 Huffman-shaped construction ({key}).",
                                          cls(dt, tree))


_register_all()


class DeviceStructure:
    """A device-resident build (pwmgpu_wx): matrix and/or tree, optional
    rank/select support, batched queries."""

    def __init__(self, size, word_width, levels, matrix=True, tree=False, rank_select=False, context=None,
                 keep_histogram=False):
        self.ctx = context or default_context()
        flags = (MATRIX if matrix else 0) | (TREE if tree else 0) | (RANK_SELECT if rank_select else 0) | \
            (KEEP_HISTOGRAM if keep_histogram else 0)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.pwmgpu_wx_create(self.ctx.h, int(size), int(word_width), int(levels), flags,
                                                     ctypes.byref(h)))
        self.h = h
        self.size, self.word_width, self.levels = int(size), int(word_width), int(levels)
        self.matrix, self.tree, self.rank_select = matrix, tree, rank_select

    @classmethod
    def huffman(cls, d_text_ptr, size, word_width, tree=False, rank_select=True, codes=None, context=None):
        """A Huffman-shaped matrix or tree built from a device text
        (pwmgpu_wx_build_huffman); codes: (code_len, code_word) u64 arrays,
        or None for pwm's builder.  Queries walk the symbols' codes."""
        self = cls.__new__(cls)
        self.ctx = context or default_context()
        flags = (TREE if tree else MATRIX) | (RANK_SELECT if rank_select else 0)
        h = ctypes.c_void_p()
        if codes is not None:
            ln = np.ascontiguousarray(codes[0], dtype=np.uint64)
            wd = np.ascontiguousarray(codes[1], dtype=np.uint64)
            args = (_u64p(ln), _u64p(wd), ln.size)
        else:
            args = (None, None, 0)
        self.ctx.check(self.ctx.lib.pwmgpu_wx_build_huffman(self.ctx.h, ctypes.c_void_p(int(d_text_ptr)), int(size),
                                                            int(word_width), flags, *args, ctypes.byref(h)))
        self.h = h
        v = self.view(1 if tree else 0)
        self.size, self.word_width, self.levels = int(size), int(word_width), int(v.levels)
        self.matrix, self.tree, self.rank_select = not tree, tree, rank_select
        return self

    def codes(self):
        """(code_len, code_word) of a Huffman-shaped structure."""
        n = ctypes.c_uint64(0)
        self.ctx.check(self.ctx.lib.pwmgpu_wx_codes(self.h, None, None, 0, ctypes.byref(n)))
        ln = np.zeros(max(n.value, 1), dtype=np.uint64)
        wd = np.zeros(max(n.value, 1), dtype=np.uint64)
        self.ctx.check(self.ctx.lib.pwmgpu_wx_codes(self.h, _u64p(ln), _u64p(wd), n.value, ctypes.byref(n)))
        return ln[:n.value], wd[:n.value]

    def build(self, d_text_ptr):
        """Builds from a device pointer (e.g. a torch tensor's data_ptr())."""
        self.ctx.check(self.ctx.lib.pwmgpu_wx_build(self.ctx.h, self.h, ctypes.c_void_p(int(d_text_ptr))))

    def build_sharded(self, d_text_ptr, shards):
        """Builds from a device text as `shards` slices merged (pwm's wx_dd_*)."""
        self.ctx.check(self.ctx.lib.pwmgpu_wx_build_sharded(self.ctx.h, self.h, ctypes.c_void_p(int(d_text_ptr)),
                                                            int(shards)))

    def merge(self, shards):
        """This structure from built shards (DeviceStructures of consecutive
        slices, created with keep_histogram=True)."""
        arr = (ctypes.c_void_p * max(len(shards), 1))(*[s.h.value if hasattr(s.h, "value") else s.h for s in shards])
        self.ctx.check(self.ctx.lib.pwmgpu_wx_merge(self.ctx.h, arr, len(shards), self.h))

    def build_host(self, text_ptr):
        """Builds from a host pointer (pinned memory is uploaded in pieces)."""
        self.ctx.check(self.ctx.lib.pwmgpu_wx_build_host(self.ctx.h, self.h, ctypes.c_void_p(int(text_ptr))))

    def compute_host(self, text_ptr, wm_ptr=None, wm_zeros=None, wt_ptr=None):
        """Host text in, host words out (pointers to u64 arrays in the layout
        of download(); pinned arrays stream the levels back during the build).
        wm_zeros: a numpy u64 array of `levels` entries, or None."""
        lib = self.ctx.lib
        cast = lambda p: ctypes.cast(ctypes.c_void_p(int(p)), _lib.u64p) if p is not None else None
        self.ctx.check(lib.pwmgpu_wx_compute_host(self.ctx.h, self.h, ctypes.c_void_p(int(text_ptr)), cast(wm_ptr),
                                                  _u64p(wm_zeros) if wm_zeros is not None else None, cast(wt_ptr)))

    def check(self):
        self.ctx.check(self.ctx.lib.pwmgpu_wx_check(self.ctx.h, self.h))

    def view(self, which):
        v = _lib.View()
        self.ctx.check(self.ctx.lib.pwmgpu_wx_view(self.h, int(which), ctypes.byref(v)))
        return v

    def download(self, which):
        """wavelet_structure on the host (which: 0 matrix, 1 tree)."""
        v = self.view(which)
        bits = [v.level_bits[i] for i in range(v.levels)]
        bvs = bit_vectors(bits)
        zeros = np.zeros(max(v.levels, 1), dtype=np.uint64)
        self.ctx.check(self.ctx.lib.pwmgpu_wx_download(self.ctx.h, self.h, int(which), _u64p(bvs.data), _u64p(zeros)))
        return wavelet_structure(bvs, None if which else [int(z) for z in zeros[:v.levels]], bool(which))

    def rank_select_blocks(self, which, level):
        counts = np.zeros(4, dtype=np.uint64)
        lib = self.ctx.lib
        self.ctx.check(lib.pwmgpu_wx_rank_select_blocks(self.ctx.h, self.h, int(which), int(level), None, None, None,
                                                        None, _u64p(counts)))
        n0, n12, ns0, ns1 = (int(c) for c in counts)
        l0 = np.zeros(max(n0, 1), dtype=np.uint64)
        l12 = np.zeros(max(2 * n12, 1), dtype=np.uint32)
        s0 = np.zeros(max(ns0, 1), dtype=np.uint32)
        s1 = np.zeros(max(ns1, 1), dtype=np.uint32)
        self.ctx.check(lib.pwmgpu_wx_rank_select_blocks(self.ctx.h, self.h, int(which), int(level), _u64p(l0),
                                                        _u32p(l12), _u32p(s0), _u32p(s1), _u64p(counts)))
        return l0[:n0], l12[:2 * n12], s0[:ns0], s1[:ns1]

    def query(self, which, op, d_a, d_b, count, d_out):
        """Batched queries on device arrays (pointers)."""
        self.ctx.check(self.ctx.lib.pwmgpu_wx_query(self.ctx.h, self.h, int(which), int(op),
                                                    ctypes.c_void_p(int(d_a)),
                                                    ctypes.c_void_p(int(d_b)) if d_b is not None else None,
                                                    int(count), ctypes.c_void_p(int(d_out))))

    def query_batch_host(self, which, ops, a, b=None):
        """A mixed batch of queries on host arrays (pwmgpu_wx_query_batch_host):
        query i is of kind ops[i] with operands a[i], b[i]; returns the answers."""
        ops = np.ascontiguousarray(ops, dtype=np.uint8)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64) if b is not None else None
        out = np.zeros(max(a.size, 1), dtype=np.uint64)
        self.ctx.check(self.ctx.lib.pwmgpu_wx_query_batch_host(self.ctx.h, self.h, int(which), ops.ctypes.data,
                                                               a.ctypes.data, b.ctypes.data if b is not None else None,
                                                               a.size, out.ctypes.data))
        return out[:a.size]

    def free(self):
        if getattr(self, "h", None):
            self.ctx.lib.pwmgpu_wx_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Batch:
    """A batch of independent plain texts built by one CUDA graph
    (pwmgpu_batch_*): every text gets a wavelet matrix and, optionally, a
    levelwise wavelet tree, bit-identical to a single build of that text.
    The context's engine at creation decides how: the tile engine (default,
    one persistent kernel over a device work queue, tile sizes tuned per
    text class) or the warp-pass engine."""

    def __init__(self, offsets, levels, word_width=1, tree=True, levels_per_pass=2, context=None):
        self.ctx = context or default_context()
        self.offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        self.levels = np.ascontiguousarray(levels, dtype=np.uint32)
        self.count = int(self.levels.size)
        self.word_width = int(word_width)
        self.tree = bool(tree)
        h = ctypes.c_void_p()
        flags = MATRIX | (TREE if tree else 0)
        self.ctx.check(self.ctx.lib.pwmgpu_batch_create(self.ctx.h, self.count, _u64p(self.offsets),
                                                        _u32p(self.levels), self.word_width, flags,
                                                        int(levels_per_pass), ctypes.byref(h)))
        self.h = h

    def build(self, d_texts_ptr):
        self.ctx.check(self.ctx.lib.pwmgpu_batch_build(self.ctx.h, self.h, ctypes.c_void_p(int(d_texts_ptr))))

    def set_levels_per_pass(self, k):
        """Warp-pass engine: levels per pass (the tile engine takes 4)."""
        self.ctx.check(self.ctx.lib.pwmgpu_batch_set_levels_per_pass(self.h, int(k)))

    def set_tile_vectors(self, v):
        """Tile engine: tiles of v (1, 2, 4) vectors per thread for every
        text, or 0 for the size tuned per text class."""
        self.ctx.check(self.ctx.lib.pwmgpu_batch_set_tile_vectors(self.h, int(v)))

    def tile_vectors(self, index):
        """Vectors per thread text `index` was built with (0: warp engine)."""
        v = ctypes.c_uint32(0)
        self.ctx.check(self.ctx.lib.pwmgpu_batch_tile_vectors(self.h, int(index), ctypes.byref(v)))
        return v.value

    def check(self):
        self.ctx.check(self.ctx.lib.pwmgpu_batch_check(self.ctx.h, self.h))

    def download(self, index, which=0):
        n = int(self.offsets[index + 1] - self.offsets[index])
        L = int(self.levels[index])
        bvs = bit_vectors([n] * L)
        zeros = np.zeros(max(L, 1), dtype=np.uint64)
        self.ctx.check(self.ctx.lib.pwmgpu_batch_download(self.ctx.h, self.h, int(index), int(which), _u64p(bvs.data),
                                                          _u64p(zeros)))
        return wavelet_structure(bvs, None if which else [int(z) for z in zeros[:L]], bool(which))

    def free(self):
        if getattr(self, "h", None):
            self.ctx.lib.pwmgpu_batch_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def generate_batch(seed, count):
    """Seeded batch of 8-bit texts (pwmgpu_generate_batch): (texts, offsets, levels)."""
    lib = _lib.load()
    offs = np.zeros(count + 1, dtype=np.uint64)
    levels = np.zeros(max(count, 1), dtype=np.uint32)
    st = lib.pwmgpu_generate_batch(int(seed), int(count), _u64p(offs), _u32p(levels), None)
    if st != 0:
        raise PwmGpuError(st, "pwmgpu_generate_batch failed")
    texts = np.zeros(max(int(offs[-1]), 1), dtype=np.uint8)
    st = lib.pwmgpu_generate_batch(int(seed), int(count), _u64p(offs), _u32p(levels), texts.ctypes.data)
    if st != 0:
        raise PwmGpuError(st, "pwmgpu_generate_batch failed")
    return texts[:int(offs[-1])], offs, levels[:count]


class Server:
    """pwmgpu_server: continuous batching of construction and query requests
    over device-resident structures, admitted under an HBM budget."""

    def __init__(self, budget_bytes, slots=8, device=0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        st = self.lib.pwmgpu_server_create(int(device), int(budget_bytes), int(slots), ctypes.byref(h))
        if st != 0:
            raise PwmGpuError(st, "server_create failed")
        self.h = h
        self._keep = {}  # host arrays that must outlive their requests

    def _check(self, st, rid=None):
        if st != 0:
            msg = self.lib.pwmgpu_server_error(self.h, int(rid)).decode() if rid is not None else ""
            raise PwmGpuError(st, msg)

    def submit(self, text, levels, matrix=True, tree=False, which=0, ops=None, a=None, b=None):
        """Build request for a host numpy text (uint8/16/32) with an optional
        query batch (ops: uint8 kinds, a/b: uint64 operands).  Returns (id,
        results array filled once the request is done)."""
        text = np.ascontiguousarray(text)
        nq = 0 if ops is None else len(ops)
        ops = np.ascontiguousarray(ops, dtype=np.uint8) if nq else None
        a = np.ascontiguousarray(a, dtype=np.uint64) if nq else None
        b = np.ascontiguousarray(b, dtype=np.uint64) if (nq and b is not None) else None
        res = np.zeros(max(nq, 1), dtype=np.uint64)
        r = _lib.Request()
        r.text = text.ctypes.data
        r.size = text.size
        r.word_width = text.dtype.itemsize
        r.levels = int(levels)
        r.shape_flags = (MATRIX if matrix else 0) | (TREE if tree else 0)
        r.query_structure = int(which)
        r.nqueries = nq
        r.query_ops = ops.ctypes.data if nq else None
        r.query_a = a.ctypes.data if nq else None
        r.query_b = b.ctypes.data if b is not None else None
        r.results = res.ctypes.data
        rid = ctypes.c_uint64()
        self._check(self.lib.pwmgpu_server_submit(self.h, ctypes.byref(r), ctypes.byref(rid)))
        self._keep[rid.value] = (text, ops, a, b, res)
        return rid.value, res[:nq]

    def submit_queries(self, structure_id, ops, a, b=None, which=0):
        ops = np.ascontiguousarray(ops, dtype=np.uint8)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64) if b is not None else None
        res = np.zeros(max(len(ops), 1), dtype=np.uint64)
        rid = ctypes.c_uint64()
        self._check(self.lib.pwmgpu_server_submit_queries(
            self.h, int(structure_id), int(which), len(ops), ops.ctypes.data, a.ctypes.data,
            b.ctypes.data if b is not None else None, res.ctypes.data, ctypes.byref(rid)))
        self._keep[rid.value] = (ops, a, b, res)
        return rid.value, res[:len(ops)]

    def wait(self, rid):
        """Blocks until the request is done; returns its info (raises on error)."""
        info = _lib.RequestInfo()
        st = self.lib.pwmgpu_server_wait(self.h, int(rid), ctypes.byref(info))
        self._check(st, rid)
        return info

    def poll(self, rid):
        """Info when done, None while queued or running."""
        info = _lib.RequestInfo()
        st = self.lib.pwmgpu_server_poll(self.h, int(rid), ctypes.byref(info))
        if st == 7:
            return None
        self._check(st, rid)
        return info

    def release(self, rid):
        self._check(self.lib.pwmgpu_server_release(self.h, int(rid)))
        self._keep.pop(int(rid), None)

    def stats(self):
        st = _lib.ServerStats()
        self._check(self.lib.pwmgpu_server_stats(self.h, ctypes.byref(st)))
        return {k: int(getattr(st, k)) for k, _ in st._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.pwmgpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def generate(dist, seed, n, word_width, param=0, device_ptr=None, context=None):
    """Seeded synthetic text (host numpy array, or into a device pointer)."""
    lib = _lib.load()
    if device_ptr is None:
        out = np.zeros(int(n), dtype=_WIDTH_DTYPE[word_width])
        st = lib.pwmgpu_generate(None, int(dist), int(seed), int(param), int(n), int(word_width),
                                 out.ctypes.data if n else None, 0)
        if st != 0:
            raise PwmGpuError(st, "pwmgpu_generate failed")
        return out
    ctx = context or default_context()
    ctx.check(lib.pwmgpu_generate(ctx.h, int(dist), int(seed), int(param), int(n), int(word_width),
                                  ctypes.c_void_p(int(device_ptr)), 1))
    return None


def copy_bits(d_dst_ptr, d_src_ptr, dst_off, src_off, length, stream=None):
    """pwm's copy_bits (merge.hpp:19-190) on device arrays of 64-bit words:
    `length` bits from bit src_off of the source to bit dst_off of the
    destination; whole destination words are stored, partial ones OR-ed."""
    st = _lib.load().pwmgpu_copy_bits(ctypes.c_void_p(int(d_dst_ptr)), ctypes.c_void_p(int(d_src_ptr)), int(dst_off),
                                      int(src_off), int(length), ctypes.c_void_p(int(stream or 0)))
    if st != 0:
        raise PwmGpuError(st, "pwmgpu_copy_bits failed")


__all__ += ["copy_bits"]
