"""CPU: include/wx_gpu.hpp (the pwm-side drop-in classes) compiles against
pwm's own headers and links against libpwmgpu.so, registered through pwm's
CONSTRUCTION_REGISTER contract.  Needs the pwm source tree, named by the
PWM_REFERENCE environment variable (skipped where it is unset or absent)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("PWM_REFERENCE") or ""

PROGRAM = r'''
#include <cstdint>
#include <iostream>
#include "util/uint_t.hpp"
#include "wx_gpu.hpp"
#include "util/decode.hpp"
// pwm's registration contract, restricted to internal memory (the reference
// registry header itself needs STXXL): a type usable in CONSTRUCTION_REGISTER.
template <typename T> struct registered {
  static_assert(!T::external_in && !T::external_out && !T::stats_support && !T::is_inplace, "internal memory");
  static constexpr bool ok = T::is_parallel && T::word_width == sizeof(uint8_t);
};
static_assert(registered<wx_gpu<uint8_t, false>>::ok && registered<wx_gpu<uint8_t, true>>::ok, "");
static_assert(registered<wx_gpu_huff<uint8_t, false>>::ok, "");
// pwm registers wm_pc / wt_pc for 40-bit alphabets too (uint40_t: 5 packed bytes)
static_assert(sizeof(uint40_t) == 5 && wx_gpu<uint40_t, false>::word_width == 5, "");
int main() {
  std::vector<uint8_t> t = {3, 1, 4, 1, 5, 9, 2, 6};
  try {
    auto wm = wx_gpu<uint8_t, false>::compute(t.data(), t.size(), 4);
    auto wt = wx_gpu<uint8_t, true>::compute(t.data(), t.size(), 4);
    auto h = wx_gpu_huff<uint8_t, true>::compute(t.data(), t.size(), 0);
    std::vector<uint40_t> t40(t.begin(), t.end());
    auto w40 = wx_gpu<uint40_t, false>::compute(t40.data(), t40.size(), 4);
    std::cout << decode_wm(wm.bvs(), wm.zeros(), t.size()).size() << decode_wt(wt.bvs(), t.size()).size()
              << decode_wm(w40.bvs(), w40.zeros(), t.size()).size() << "\n";
  } catch (const std::exception& e) {
    std::cout << "runtime: " << e.what() << "\n";
    return 2;
  }
  return 0;
}
'''


@pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF, "include")),
                    reason="PWM_REFERENCE unset or not a pwm source tree")
def test_drop_in_header_compiles_and_links(tmp_path):
    src = tmp_path / "use_wx_gpu.cpp"
    src.write_text(PROGRAM)
    lib_dir = os.path.join(ROOT, "pwm_gb300")
    if not os.path.exists(os.path.join(lib_dir, "libpwmgpu.so")):
        pytest.skip("libpwmgpu.so not built")
    exe = tmp_path / "use_wx_gpu"
    cmd = ["g++", "-std=c++17", "-DNDEBUG", "-fopenmp", f"-I{os.path.join(ROOT, 'include')}",
           f"-I{os.path.join(REF, 'include')}", str(src), "-o", str(exe), f"-L{lib_dir}", "-lpwmgpu",
           f"-Wl,-rpath,{lib_dir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # without a GPU the engine reports that no device is usable (no fallback)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode in (0, 2)
    if out.returncode == 2:
        assert "no usable CUDA device" in out.stdout
