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
