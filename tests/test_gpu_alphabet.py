"""GPU: pwm's reduce_alphabet (include/util/alphabet_util.hpp:18-45) on the
device (pwmgpu_reduce_alphabet) against the oracle's restatement: symbols
renumbered by first occurrence, max_char = distinct symbols - 1."""
import numpy as np
import pytest

from conftest import text_from_hex

pytestmark = pytest.mark.gpu


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def run(pg, torch, text, in_place):
    d = torch.from_numpy(text.view(np.uint8).copy()).cuda()
    out = d if in_place else torch.empty_like(d)
    mc = pg.reduce_alphabet(d.data_ptr(), text.size, text.dtype.itemsize, out.data_ptr())
    return out.cpu().numpy().view(text.dtype), mc


@pytest.mark.parametrize("in_place", [False, True])
def test_reduce_alphabet_matches_oracle(pg, orc, in_place):
    torch = torch_cuda()
    rng = np.random.default_rng(3)
    texts = [
        rng.integers(0, 256, 1_000_003).astype(np.uint8),                      # symbol 255 included
        rng.choice(np.array([7, 200, 13], np.uint8), 5000),
        pg.generate(pg.GEN_MIX16, 2, 500_001, 2),
        rng.choice(rng.integers(0, 1 << 24, 3000).astype(np.uint32), 400_000),  # sparse 32-bit values
        np.array([9], np.uint16),
    ]
    for t in texts:
        got, mc = run(pg, torch, t, in_place)
        want, wmc = orc.reduce_alphabet(t)
        assert mc == wmc and np.array_equal(got, want), t.dtype


def test_reduce_alphabet_fixtures_and_edges(pg, orc, golden_fixtures):
    torch = torch_cuda()
    for case in golden_fixtures:
        t = text_from_hex(case["text_hex"])
        if t.size == 0:
            continue
        got, mc = run(pg, torch, t, False)
        want, wmc = orc.reduce_alphabet(t)
        assert mc == wmc and np.array_equal(got, want)
    d = torch.zeros(1, dtype=torch.uint8, device="cuda")
    assert pg.reduce_alphabet(d.data_ptr(), 0, 1) == (1 << 64) - 1  # pwm: 0 - 1


def to_u40(v):
    v = np.asarray(v, dtype=np.uint64)
    b = np.zeros((v.size, 5), np.uint8)
    for k in range(5):
        b[:, k] = ((v >> np.uint64(8 * k)) & np.uint64(0xFF)).astype(np.uint8)
    return b.reshape(-1)


@pytest.mark.parametrize("in_place", [False, True])
def test_reduce_wide_symbols(pg, orc, in_place):
    """32-bit symbols from 2^24 up and 40-bit symbols (pwm's uint40_t) go
    through a device hash table."""
    torch = torch_cuda()
    rng = np.random.default_rng(5)
    for width, top, n, distinct in ((4, 1 << 32, 1_000_003, 5000), (4, 1 << 32, 300_001, 250_000),
                                    (5, 1 << 40, 700_001, 20000), (5, 1 << 40, 3, 2)):
        vals = rng.choice(rng.integers(0, top, distinct, dtype=np.uint64), n)
        vals[0] = top - 1  # the largest value
        want, wmc = orc.reduce_alphabet(vals)
        raw = vals.astype(np.uint32).view(np.uint8) if width == 4 else to_u40(vals)
        d = torch.from_numpy(raw.copy()).cuda()
        out = d if in_place else torch.empty_like(d)
        mc = pg.reduce_alphabet(d.data_ptr(), n, width, out.data_ptr())
        got = out.cpu().numpy()
        expect = want.astype(np.uint32).view(np.uint8) if width == 4 else to_u40(want)
        assert mc == wmc and np.array_equal(got, expect), (width, n)


def test_reduce_alphabet_matches_pwm_golden(pg):
    """Against pwm's own reduce_alphabet (tests/golden/alphabet.json, recorded
    by running pwm's function on the shared generator's texts)."""
    import hashlib
    import json
    import os
    from conftest import GOLDEN
    torch = torch_cuda()
    with open(os.path.join(GOLDEN, "alphabet.json")) as f:
        cases = json.load(f)["cases"]
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a, a.dtype.newbyteorder("<")).tobytes()).hexdigest()
    for c in cases:
        t = pg.generate(c["dist"], c["seed"], c["n"], c["width"], param=c["param"])
        assert sha(t) == c["text_sha256"], c["name"]
        got, mc = run(pg, torch, t, False)
        assert mc == c["max_char"], c["name"]
        assert sha(got) == c["out_sha256"], c["name"]
