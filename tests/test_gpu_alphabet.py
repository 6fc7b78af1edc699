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
    big = torch.from_numpy(np.array([1 << 24, 3], np.uint32).view(np.uint8)).cuda()
    with pytest.raises(pg.PwmGpuError):
        pg.reduce_alphabet(big.data_ptr(), 2, 4)
