"""Loads libpwmgpu.so (built in-tree by pwm_gb300/build.py) and declares the
C ABI of include/pwmgpu.h.  There is no fallback: if the library is missing
or no GB300 is usable, calls fail with an error."""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpwmgpu.so")
HEADER = os.path.join(HERE, "..", "include", "pwmgpu.h")

u64 = ctypes.c_uint64
u32 = ctypes.c_uint32
i32 = ctypes.c_int
vp = ctypes.c_void_p
u64p = ctypes.POINTER(ctypes.c_uint64)
u32p = ctypes.POINTER(ctypes.c_uint32)
cstr = ctypes.c_char_p

STATUS = {0: "PWMGPU_OK", 1: "PWMGPU_ERR_ARG", 2: "PWMGPU_ERR_OOM", 3: "PWMGPU_ERR_CUDA",
          4: "PWMGPU_ERR_TIMEOUT", 5: "PWMGPU_ERR_SYMBOL", 6: "PWMGPU_ERR_NO_DEVICE", 7: "PWMGPU_ERR_BUSY"}

MATRIX, TREE, RANK_SELECT, HUFFMAN, KEEP_HISTOGRAM = 0x1, 0x2, 0x4, 0x8, 0x10
Q_ACCESS, Q_RANK, Q_SELECT = 0, 1, 2
GEN_UNIFORM, GEN_DNA4, GEN_ZIPF256, GEN_MIX16 = 0, 1, 2, 3


class View(ctypes.Structure):
    _fields_ = [("levels", u32), ("is_tree", u32), ("is_huffman", u32), ("has_rank_select", u32),
                ("size", u64), ("total_words", u64), ("words", vp), ("level_offset", u64p),
                ("level_bits", u64p), ("zeros", u64p)]


class Request(ctypes.Structure):
    _fields_ = [("text", vp), ("size", u64), ("word_width", u32), ("levels", u32), ("shape_flags", u32),
                ("query_structure", u32), ("nqueries", u64), ("query_ops", vp), ("query_a", vp),
                ("query_b", vp), ("results", vp)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("id", u64), ("status", i32), ("slot", u32), ("submit_s", ctypes.c_double),
                ("start_s", ctypes.c_double), ("done_s", ctypes.c_double), ("device_bytes", u64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("budget_bytes", u64), ("in_use_bytes", u64), ("peak_bytes", u64), ("queued", u64),
                ("running", u64), ("completed", u64)]


# name -> (restype, argtypes)
SIGNATURES = {
    "pwmgpu_ctx_create": (i32, [i32, vp, ctypes.POINTER(vp)]),
    "pwmgpu_ctx_destroy": (None, [vp]),
    "pwmgpu_ctx_last_error": (cstr, [vp]),
    "pwmgpu_status_string": (cstr, [i32]),
    "pwmgpu_ctx_sync": (i32, [vp]),
    "pwmgpu_ctx_launch_count": (u64, [vp]),
    "pwmgpu_ctx_set_pass_levels": (i32, [vp, i32]),
    "pwmgpu_ctx_set_engine": (i32, [vp, i32]),
    "pwmgpu_ctx_profile": (i32, [vp, i32]),
    "pwmgpu_ctx_profile_read": (i32, [vp, ctypes.c_char_p, u64]),
    "pwmgpu_wx_build_host": (i32, [vp, vp, vp]),
    "pwmgpu_wx_compute_host": (i32, [vp, vp, vp, u64p, u64p, u64p]),
    "pwmgpu_wx_merge": (i32, [vp, ctypes.POINTER(vp), u32, vp]),
    "pwmgpu_wx_build_sharded": (i32, [vp, vp, vp, u32]),
    "pwmgpu_copy_bits": (i32, [vp, vp, u64, u64, u64, vp]),
    "pwmgpu_ctx_set_upload_piece_bytes": (i32, [vp, u64]),
    "pwmgpu_ctx_set_host_copy_threads": (i32, [vp, i32]),
    "pwmgpu_ctx_set_stream_chunks": (i32, [vp, u32]),
    "pwmgpu_ctx_set_spin_limit": (i32, [vp, u32]),
    "pwmgpu_ctx_test_withhold_tile": (i32, [vp, i32]),
    "pwmgpu_ctx_release_scratch": (i32, [vp]),
    "pwmgpu_wx_build_huffman": (i32, [vp, vp, u64, u32, u32, u64p, u64p, u64, ctypes.POINTER(vp)]),
    "pwmgpu_wx_codes": (i32, [vp, u64p, u64p, u64, u64p]),
    "pwmgpu_compute_semi_external": (i32, [vp, vp, u64, u32, u32, u64p, u64p, u64p, u64]),
    "pwmgpu_reduce_alphabet": (i32, [vp, vp, u64, u32, vp, u64p]),
    "pwmgpu_compute": (i32, [vp, vp, u64, u32, u32, i32, u64p, u64p]),
    "pwmgpu_huffman_codes": (i32, [vp, vp, u64, u32, i32, u64p, u64p, u64, u64p, u64p, u32p]),
    "pwmgpu_compute_huffman": (i32, [vp, vp, u64, u32, i32, u64p, u64p, u64, u32, u64p, u64p, u64p]),
    "pwmgpu_wx_create": (i32, [vp, u64, u32, u32, u32, ctypes.POINTER(vp)]),
    "pwmgpu_wx_build": (i32, [vp, vp, vp]),
    "pwmgpu_wx_check": (i32, [vp, vp]),
    "pwmgpu_wx_view": (i32, [vp, i32, ctypes.POINTER(View)]),
    "pwmgpu_wx_download": (i32, [vp, vp, i32, u64p, u64p]),
    "pwmgpu_wx_rank_select_blocks": (i32, [vp, vp, i32, u32, u64p, u32p, u32p, u32p, u64p]),
    "pwmgpu_wx_query": (i32, [vp, vp, i32, i32, vp, vp, u64, vp]),
    "pwmgpu_wx_free": (None, [vp]),
    "pwmgpu_wx_query_host": (i32, [vp, vp, i32, i32, vp, vp, u64, vp]),
    "pwmgpu_wx_query_batch_host": (i32, [vp, vp, i32, vp, vp, vp, u64, vp]),
    "pwmgpu_ctx_set_stream_ordered_alloc": (i32, [vp, i32]),
    "pwmgpu_server_create": (i32, [i32, u64, u32, ctypes.POINTER(vp)]),
    "pwmgpu_server_submit": (i32, [vp, ctypes.POINTER(Request), u64p]),
    "pwmgpu_server_submit_queries": (i32, [vp, u64, u32, u64, vp, vp, vp, vp, u64p]),
    "pwmgpu_server_wait": (i32, [vp, u64, ctypes.POINTER(RequestInfo)]),
    "pwmgpu_server_poll": (i32, [vp, u64, ctypes.POINTER(RequestInfo)]),
    "pwmgpu_server_error": (cstr, [vp, u64]),
    "pwmgpu_server_release": (i32, [vp, u64]),
    "pwmgpu_server_stats": (i32, [vp, ctypes.POINTER(ServerStats)]),
    "pwmgpu_server_destroy": (None, [vp]),
    "pwmgpu_generate": (i32, [vp, i32, u64, u64, u64, u32, vp, i32]),
    "pwmgpu_batch_create": (i32, [vp, u32, u64p, u32p, u32, u32, i32, ctypes.POINTER(vp)]),
    "pwmgpu_batch_build": (i32, [vp, vp, vp]),
    "pwmgpu_batch_set_levels_per_pass": (i32, [vp, i32]),
    "pwmgpu_batch_set_tile_vectors": (i32, [vp, u32]),
    "pwmgpu_batch_tile_vectors": (i32, [vp, u32, u32p]),
    "pwmgpu_batch_check": (i32, [vp, vp]),
    "pwmgpu_batch_download": (i32, [vp, vp, u32, i32, u64p, u64p]),
    "pwmgpu_batch_free": (None, [vp]),
    "pwmgpu_generate_batch": (i32, [u64, u32, u64p, u32p, vp]),
    "pwmgpu_rank_select_build_noalloc": (i32, [vp, u64, vp, vp, vp, vp, vp, vp]),
}


class PwmGpuError(RuntimeError):
    def __init__(self, status, message=""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {message}")


_lib = None


def load():
    """Returns the loaded library; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                           "(nvcc, sm_103a) first; this package has no CPU fallback")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def declared_symbols():
    """Entry points declared in include/pwmgpu.h."""
    import re
    text = open(HEADER).read()
    return sorted(set(re.findall(r"PWMGPU_API\s+[\w\s\*]+?\b(pwmgpu_\w+)\s*\(", text)))
