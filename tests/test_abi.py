"""CPU: the C-ABI library loads and exports every entry point declared in
include/pwmgpu.h; host-side calls that need no GPU behave."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from pwm_gb300 import _lib


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from pwm_gb300 import build
        build.build()
    return _lib.load()


def test_header_declares_entry_points():
    syms = _lib.declared_symbols()
    for name in ("pwmgpu_compute", "pwmgpu_compute_huffman", "pwmgpu_huffman_codes", "pwmgpu_wx_create",
                 "pwmgpu_wx_build", "pwmgpu_wx_query", "pwmgpu_wx_rank_select_blocks", "pwmgpu_ctx_create"):
        assert name in syms


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {line.split()[-1] for line in out.stdout.splitlines() if line.strip()}
    missing = [s for s in _lib.declared_symbols() if s not in exported]
    assert not missing, missing
    for s in _lib.declared_symbols():
        assert hasattr(lib, s)
    # nothing but the C ABI is exported
    assert all(e.startswith("pwmgpu_") or e.startswith("_") for e in exported if not e.startswith("__"))


def test_python_binding_covers_the_header():
    assert set(_lib.declared_symbols()) <= set(_lib.SIGNATURES)


def test_status_strings(lib):
    for st in range(8):
        assert lib.pwmgpu_status_string(st)


def test_null_arguments_are_rejected(lib):
    assert lib.pwmgpu_ctx_create(0, None, None) == 1
    assert lib.pwmgpu_compute(None, None, 0, 1, 8, 0, None, None) == 1
    assert lib.pwmgpu_generate(None, 0, 1, 4, 10, 3, None, 0) == 1  # width 3


def test_host_generator_is_deterministic(lib):
    import pwm_gb300 as pg
    a = pg.generate(pg.GEN_ZIPF256, 5, 10_000, 1)
    b = pg.generate(pg.GEN_ZIPF256, 5, 10_000, 1)
    c = pg.generate(pg.GEN_ZIPF256, 6, 10_000, 1)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    d = pg.generate(pg.GEN_DNA4, 1, 200_000, 1)
    freq = np.bincount(d, minlength=4) / d.size
    assert np.allclose(freq, [0.3, 0.2, 0.2, 0.3], atol=0.01)
    m = pg.generate(pg.GEN_MIX16, 1, 200_000, 2)
    assert (m < 2000).mean() > 0.5  # the geometric half is concentrated on small ids
    u = pg.generate(pg.GEN_UNIFORM, 1, 100_000, 4, param=1 << 20)
    assert u.max() < (1 << 20)


def test_header_compiles_as_c(tmp_path):
    """include/pwmgpu.h is a C header (plain types, C linkage): a C99 program
    that takes the address of every declared entry point compiles cleanly."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    refs = "\n".join("  (void)&%s;" % s for s in _lib.declared_symbols())
    src = tmp_path / "use_abi.c"
    src.write_text('#include "pwmgpu.h"\nint main(void) {\n%s\n  return 0;\n}\n' % refs)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-c",
                        f"-I{os.path.join(root, 'include')}", str(src), "-o", str(tmp_path / "use_abi.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
