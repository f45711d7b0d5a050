"""The bit-mask form of the pattern rank used by the engine's kernels
(ga_problems.cuh PuzzleProblem::rank, pdb.cu decode) restated in Python and
checked against the oracle's restatement of the reference's encoding
(src/puzzle/database.cpp:140-199).  CPU only."""
from __future__ import annotations

import numpy as np

import oracle as O


def mults(n, k):
    return [int(np.prod([n * n - i for i in range(j, k)], dtype=np.int64)) for j in range(k + 1)]


def rank_bitmask(n, tracked, conf):
    pos = {t: i for i, t in enumerate(conf) if t}
    m = mults(n, len(tracked))
    used, code = 0, 0
    for j, t in enumerate(tracked):
        p = pos[t]
        v = p - bin(used & ((1 << p) - 1)).count("1")
        code += v * m[j + 1]
        used |= 1 << p
    return code


def decode_bitmask(n, tracked, code):
    m = mults(n, len(tracked))
    used = 0
    conf = [0] * (n * n)
    for j, t in enumerate(tracked):
        v = code // m[j + 1]
        code -= v * m[j + 1]
        # the v-th (0-based) cell not used by earlier tiles (__fns(~used, 0, v+1))
        free = [c for c in range(32) if not (used >> c) & 1]
        cell = free[v]
        conf[cell] = t
        used |= 1 << cell
    return conf


def test_multipliers_match_reference_table():
    # the multiplier rows the reference's GPU kernel hard-codes (GPU-kernel.cuh:74-79)
    assert mults(3, 8) == [362880, 40320, 5040, 720, 120, 24, 6, 2, 1]
    assert mults(4, 8) == [518918400, 32432400, 2162160, 154440, 11880, 990, 90, 9, 1]
    assert mults(4, 7) == [57657600, 3603600, 240240, 17160, 1320, 110, 10, 1]


def test_bitmask_rank_equals_reference_encoding():
    rng = np.random.default_rng(7)
    for n, parts in O.PARTITIONS.items():
        for tracked in parts:
            for _ in range(300):
                perm = rng.permutation(n * n)
                conf = [int(t) if int(t) in tracked else 0 for t in perm]
                assert rank_bitmask(n, tracked, conf) == O.pattern_encode(n, tracked, conf)


def test_bitmask_decode_equals_reference_decoding():
    rng = np.random.default_rng(8)
    for n, parts in O.PARTITIONS.items():
        for tracked in parts:
            size = O.pattern_size(n, tracked)
            for code in rng.integers(0, size, 300):
                assert decode_bitmask(n, tracked, int(code)) == O.pattern_decode(n, tracked, int(code)).tolist()


def test_goal_rank():
    for n, parts in O.PARTITIONS.items():
        for tracked in parts:
            conf = [0] * (n * n)
            for t in tracked:
                conf[t - 1] = t
            assert rank_bitmask(n, tracked, conf) == O.pattern_encode(n, tracked, conf)
