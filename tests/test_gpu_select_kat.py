"""GPU: pwm's own select test (test/bin_rank_select_tests.cpp:38-61) through
this library's rank/select support: the 2^27-bit vector of std::mt19937(44227)
words (tests/host_logic/mt_bits.cpp, generated with the C++ standard library
as pwm's test does; its hash recorded here) is level 0 of a one-level wavelet
matrix over the text of its bits, so select of symbol 1 / 0 is select1 /
select0 of the vector.  As in pwm's test, every position of the first 1% is
checked (select1 at each one, select0 at each zero), and rank (pwm's
commented-out test, :17-36) at every 97th position of the vector."""
import hashlib
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "host_logic", "mt_bits.cpp")
SHA = "842ba359ba7d282f36b9c06ae6ac2237b7f047f38abe4504403435a18fe22311"


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def query(ds, op, a, b):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    b = np.ascontiguousarray(b, dtype=np.uint64)
    out = np.zeros(a.size, dtype=np.uint64)
    ds.ctx.check(ds.ctx.lib.pwmgpu_wx_query_host(ds.ctx.h, ds.h, 0, op, a.ctypes.data, b.ctypes.data, a.size,
                                                 out.ctypes.data))
    return out


def test_pwm_select_known_answers(pg, tmp_path):
    torch = torch_cuda()
    exe, path = str(tmp_path / "mt_bits"), str(tmp_path / "bits.bin")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-o", exe, SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([exe, path]).returncode == 0
    words = np.fromfile(path, dtype="<u8")
    assert hashlib.sha256(words.tobytes()).hexdigest() == SHA
    bits = np.unpackbits(words.astype(">u8").view(np.uint8))  # bit i: bit 63 - i%64 of word i/64
    n = bits.size
    assert n == 1 << 27
    d = torch.from_numpy(bits).cuda()
    ds = pg.DeviceStructure(n, 1, 1, matrix=True, rank_select=True)
    ds.build(d.data_ptr())
    ds.check()
    assert np.array_equal(np.asarray(ds.download(0).bvs()[0]), words)  # level 0 is the vector
    head = bits[:n // 100].astype(np.int64)
    ones_through = np.cumsum(head)
    pos = np.arange(head.size, dtype=np.uint64)
    one = head == 1
    # select1(one_count) == i at every one, select0(i - one_count + 1) == i at every zero
    got1 = query(ds, pg.Q_SELECT, np.ones(int(one.sum()), np.uint64), ones_through[one])
    assert np.array_equal(got1, pos[one])
    zeros_through = np.arange(1, head.size + 1) - ones_through
    got0 = query(ds, pg.Q_SELECT, np.zeros(int((~one).sum()), np.uint64), zeros_through[~one])
    assert np.array_equal(got0, pos[~one])
    # rank1 / rank0 at every 97th position of the whole vector
    idx = np.arange(0, n + 1, 97, dtype=np.uint64)
    before = np.concatenate([[0], np.cumsum(bits.astype(np.int64))])[idx.astype(np.int64)]
    assert np.array_equal(query(ds, pg.Q_RANK, np.ones(idx.size, np.uint64), idx), before.astype(np.uint64))
    assert np.array_equal(query(ds, pg.Q_RANK, np.zeros(idx.size, np.uint64), idx), (idx - before).astype(np.uint64))
    ds.free()
