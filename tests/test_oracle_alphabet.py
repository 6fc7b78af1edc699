"""CPU: the oracle's restatement of pwm's reduce_alphabet
(include/util/alphabet_util.hpp:18-45) on hand-checked cases."""
import numpy as np


def test_reduce_alphabet_restatement(orc):
    t, mc = orc.reduce_alphabet(np.array([5, 3, 5, 7, 3, 255], np.uint8))
    assert t.tolist() == [0, 1, 0, 2, 1, 3] and mc == 3
    t, mc = orc.reduce_alphabet(np.array([40000, 2, 40000], np.uint16))
    assert t.tolist() == [0, 1, 0] and t.dtype == np.uint16 and mc == 1
    t, mc = orc.reduce_alphabet(np.zeros(0, np.uint32))
    assert t.size == 0 and mc == (1 << 64) - 1


def test_reduce_alphabet_restatement_matches_pwm_golden(orc):
    """The restatement against pwm's own reduce_alphabet
    (tests/golden/alphabet.json)."""
    import hashlib
    import json
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "alphabet.json")) as f:
        cases = json.load(f)["cases"]
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a, a.dtype.newbyteorder("<")).tobytes()).hexdigest()
    for c in cases:
        t = orc.generate(c["dist"], c["seed"], c["n"], c["width"], param=c["param"])
        assert sha(t) == c["text_sha256"], c["name"]
        out, mc = orc.reduce_alphabet(t)
        assert mc == c["max_char"] and sha(out) == c["out_sha256"], c["name"]
