"""pwm's side of the boundary, run: the registration unit a pwm maintainer adds
(integration/gpu_construction.cpp, pwm's CONSTRUCTION_REGISTER pattern) and
the drop-in classes of include/wx_gpu.hpp, compiled into a program with
stand-ins for the pwm interface they use (tests/pwm_standin/; pwm's own tree
is not on GPU hosts) and linked against libpwmgpu.so.

CPU: the program builds and registers every construction with pwm's static
traits.  GPU: every registered construction (wm_gpu / wt_gpu for 8-, 16-,
32- and 40-bit alphabets, wm_gpu_huff / wt_gpu_huff for 8 and 16 bits) is
run through the registry on seeded texts, and the returned wavelet_structure
(every level word, the level sizes and the matrix zeros) must equal pwm's own
output recorded in tests/golden/seeded.json.  Integer data: exact equality.
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "pwm_gb300")


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not os.path.exists(os.path.join(LIB_DIR, "libpwmgpu.so")):
        from pwm_gb300 import build
        build.build()
    exe = str(tmp_path_factory.mktemp("dropin") / "run_registered")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", f"-I{os.path.join(ROOT, 'tests', 'pwm_standin')}",
           f"-I{os.path.join(ROOT, 'include')}", os.path.join(ROOT, "integration", "gpu_construction.cpp"),
           os.path.join(ROOT, "tests", "pwm_standin", "run_registered.cpp"), "-o", exe, f"-L{LIB_DIR}", "-lpwmgpu",
           f"-Wl,-rpath,{LIB_DIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_registration_unit_registers_every_width(driver):
    out = subprocess.run([driver, "list"], capture_output=True, text=True, check=True).stdout.split("\n")
    regs = {}
    for line in filter(None, out):
        name, w, tree, huff, par, ein, eout, stats, inplace = line.split()
        regs[(name, int(w))] = (int(tree), int(huff), int(par), int(ein), int(eout), int(stats), int(inplace))
    expect = {("wm_gpu", w): (0, 0) for w in (1, 2, 4, 5)}
    expect.update({("wt_gpu", w): (1, 0) for w in (1, 2, 4, 5)})
    expect.update({("wm_gpu_huff", w): (0, 1) for w in (1, 2)})
    expect.update({("wt_gpu_huff", w): (1, 1) for w in (1, 2)})
    assert set(regs) == set(expect)
    for k, (tree, huff) in expect.items():
        # pwm's registry contract: internal memory, parallel, no stats, not in place
        assert regs[k] == (tree, huff, 1, 0, 0, 0, 0), k


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def _run(driver, tmp_path, name, width, levels, text_bytes):
    src, dst = tmp_path / "text.bin", tmp_path / "out.bin"
    src.write_bytes(text_bytes)
    r = subprocess.run([driver, name, str(width), str(levels), str(src), str(dst)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, (name, width, r.stdout, r.stderr)
    raw = np.fromfile(dst, dtype="<u8")
    L = int(raw[0])
    bits = [int(b) for b in raw[1:1 + L]]
    nz = int(raw[1 + L])
    zeros = [int(z) for z in raw[2 + L:2 + L + nz]]
    words, off = [], 2 + L + nz
    for b in bits:
        k = (b + 63) // 64
        words.append(raw[off:off + k])
        off += k
    return bits, zeros, words


def _check(got, golden, label):
    bits, zeros, words = got
    assert bits == golden["level_bits"], label
    assert [_sha(w) for w in words] == golden["sha256"], label
    if golden["zeros"] is not None:
        assert zeros == golden["zeros"], label
    else:
        assert zeros == [], label


CASES = [  # (golden case, widths of the plain registrations to run on it)
    ("dna4_l2", (1,)),
    ("zipf256_l8", (1,)),
    ("mix16_l16", (2,)),
    ("uniform_u32_l20", (4, 5)),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case_name,widths", CASES)
def test_registered_constructions_match_pwm(driver, golden_seeded, pg, tmp_path, case_name, widths):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    case = next(c for c in golden_seeded if c["name"] == case_name)
    text = pg.generate(case["dist"], case["seed"], case["n"], case["width"], param=case["param"])
    for w in widths:
        if w == 5:  # pwm's uint40_t: five bytes per symbol, little endian
            raw = np.zeros((text.size, 8), np.uint8)
            raw[:] = text.astype("<u8").view(np.uint8).reshape(-1, 8)
            payload = raw[:, :5].tobytes()
        else:
            payload = text.tobytes()
        for name, key in (("wm_gpu", "wm"), ("wt_gpu", "wt")):
            _check(_run(driver, tmp_path, name, w, case["levels"], payload), case[key], f"{name}/{w}")
    if case["width"] <= 2:
        for name, key in (("wm_gpu_huff", "wm_huff"), ("wt_gpu_huff", "wt_huff")):
            _check(_run(driver, tmp_path, name, case["width"], 0, text.tobytes()), case[key],
                   f"{name}/{case['width']}")
