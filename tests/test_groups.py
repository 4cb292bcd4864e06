"""Target groups of the pair kernels by key-block bisection (csrc/tree.cu: group_start).

The groups are the largest aligned key blocks (one key bit at a time) holding at most G particles
of one run, with runs of more than G equal keys cut every G particles.  The device forms them
from one local predicate per particle (does particle i start a group?) instead of a recursive
split; these tests restate that predicate here and check it against the recursive definition on
key sets with runs, duplicate keys and depth-capped (zero-filled) low bits."""
import numpy as np
import pytest


def group_start(keys, run, G, i):
    """Host restatement of the device predicate (csrc/tree.cu: group_start), step for step."""
    n = len(keys)
    if i == 0 or run[i] != run[i - 1]:
        return True
    ki = int(keys[i])
    x = int(keys[i - 1]) ^ ki
    L = 64 - x.bit_length()
    mask = (1 << 64) - 1 if L >= 64 else (0 if L == 0 else (((1 << 64) - 1) << (64 - L)) & ((1 << 64) - 1))
    lo = i - 1 - G
    if lo >= 0 and ((int(keys[lo]) ^ ki) & mask) == 0:
        if x != 0:
            return True
        a, b = 0, lo
        while a < b:
            m = (a + b) >> 1
            if int(keys[m]) == ki:
                b = m
            else:
                a = m + 1
        return (i - a) % G == 0
    a, b = max(lo + 1, 0), i - 1
    while a < b:
        m = (a + b) >> 1
        if ((int(keys[m]) ^ ki) & mask) == 0:
            b = m
        else:
            a = m + 1
    if not (a + G < n and ((int(keys[a + G]) ^ ki) & mask) == 0):
        return False
    return x != 0 or (i - a) % G == 0


def bisect_groups(keys, run, G):
    """The definition: split [b, e) at its highest key bit while it holds more than G particles;
    equal keys are cut every G particles; runs are never merged."""
    out = []
    n = len(keys)
    starts = [0] + [i for i in range(1, n) if run[i] != run[i - 1]] + [n]

    def rec(b, e, bit):
        if e - b <= G:
            out.append((b, e - b))
            return
        if bit < 0:
            for s in range(b, e, G):
                out.append((s, min(G, e - s)))
            return
        m = b
        while m < e and not ((int(keys[m]) >> bit) & 1):
            m += 1
        if m > b:
            rec(b, m, bit - 1)
        if e > m:
            rec(m, e, bit - 1)

    for r in range(len(starts) - 1):
        rec(starts[r], starts[r + 1], 63)
    return out


def groups_from_predicate(keys, run, G):
    n = len(keys)
    flags = [group_start(keys, run, G, i) for i in range(n)]
    pos = [i for i in range(n) if flags[i]] + [n]
    return [(pos[k], pos[k + 1] - pos[k]) for k in range(len(pos) - 1)]


@pytest.mark.parametrize("seed", range(8))
@pytest.mark.parametrize("G", [1, 4, 32])
def test_predicate_equals_recursive_bisection(seed, G):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 400))
    nruns = int(rng.integers(1, 4))
    run = np.sort(rng.integers(0, nruns, n))
    # keys: run index on top, then digits; few distinct low patterns so that equal keys and
    # clusters occur; some sets keep only the top digits (a depth-capped build)
    digits = rng.integers(0, 1 << 12, n) if seed % 2 else rng.integers(0, 64, n) << 6
    if seed % 3 == 0:
        digits = (rng.integers(0, 4, n) << 10) | rng.integers(0, 3, n)
    keys = (run.astype(np.uint64) << np.uint64(60)) | digits.astype(np.uint64)
    order = np.lexsort((keys,))
    keys, run = keys[order], run[order]
    got = groups_from_predicate(keys, run, G)
    want = bisect_groups(keys, run, G)
    assert got == want
    assert all(1 <= c <= G for _, c in got)


def test_long_equal_key_runs_are_cut_every_G():
    keys = np.array([5] * 70 + [6] * 3 + [7] * 33, dtype=np.uint64)
    run = np.zeros(len(keys), dtype=np.int64)
    got = groups_from_predicate(keys, run, 32)
    assert got == bisect_groups(keys, run, 32)
    assert got[:3] == [(0, 32), (32, 32), (64, 6)]
