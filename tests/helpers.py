"""Helpers shared by the test modules."""
import hashlib

import numpy as np


def sha_words(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def sha_u32(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u4").tobytes()).hexdigest()


def seeded_text(pg, case):
    return pg.generate(case["dist"], case["seed"], case["n"], case["width"], param=case["param"])


def level_words(ws, l):
    """Meaningful words of level l of a pwm_gb300.wavelet_structure."""
    return np.asarray(ws.bvs()[l])


def brute_rank(text, sym, i):
    return int(np.count_nonzero(text[:i] == sym))


def brute_select(text, sym, occ):
    pos = np.nonzero(text == sym)[0]
    return int(pos[occ - 1])
