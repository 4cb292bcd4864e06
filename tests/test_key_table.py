"""Host restatements of two exactness arguments of the device code, checked on the CPU with IEEE
FP64 / FP32 numpy arithmetic (no GPU):

1. The octree key table (csrc/tree.cu: key_table_kernel, keys_kernel).  The digits of a
   particle's key are the path of the reference's centre recursion (BHTree::make's child centres,
   src/bhtree.cpp:190-196): at each level compare x > c per axis, then move c by +/- edge/4,
   edge/8, ... (one FP64 rounding per move).  The device replays the first T levels once per node
   of a complete binary tree (heap order) and searches that table with integer comparisons of the
   ordered-integer images, then continues the recursion from the level-T centre.  The test
   restates both procedures step for step (including the exponent-field arithmetic that forms
   edge * 2^-(l+2)) and checks that they give the same digits, on centres and edges of all scales,
   coordinates equal to centres, signed zeros and coordinates outside the root box.

2. The FP32 pre-pass of TimeStep's force minimum (csrc/integrate.cu: dt_estimate): for h and the
   largest |a_k| in [2^-60, 2^60], the FP32 estimate of sqrt(h / |a|) is within 4 * 2^-24 of the
   exact value (the device uses the bound 2^-21 and a candidate margin of 2^-12)."""
import numpy as np
import pytest

MASK52 = np.int64(1) << np.int64(52)


def ord_image(x):
    """Ordered-integer image of a double (the device's dbl_to_ord)."""
    i = np.float64(x).view(np.int64)
    return i if i >= 0 else np.int64(i ^ np.int64(0x7FFFFFFFFFFFFFFF))


def q_sequence(e0, levels):
    """edge * 2^-(l+2) for l = 0 .. levels-1 as the device forms them: the exponent field of the
    edge decremented (an integer subtraction on the bits); 0 for a zero-extent root."""
    if not e0 > 0.0:
        return [0.0] * levels
    qb = np.float64(e0).view(np.int64) - (np.int64(2) << np.int64(52))
    out = []
    for _ in range(levels):
        out.append(float(np.int64(qb).view(np.float64)))
        qb = qb - MASK52
    return out


def digits_recursion(x, c0, e0, levels):
    """The recursion of keys_kernel without a table: per level the comparison on ordered images and
    one rounded FP64 move of the centre."""
    c = float(np.float64(c0) + 0.0)
    xo = ord_image(x + 0.0)
    qs = q_sequence(e0, levels)
    out = []
    for l in range(levels):
        up = xo > ord_image(c)
        out.append(1 if up else 0)
        c = float(np.float64(c) + np.float64(qs[l] if up else -qs[l]))
    return out


def build_table(c0, e0, T):
    """key_table_kernel for one axis: entry k (1 <= k < 2^(T+1)) replays its heap path; entries of
    depth < T hold ordered images, those of depth T the centre itself."""
    qs = q_sequence(e0, T)
    table = [None] * (2 << T)
    for k in range(1, 2 << T):
        depth = k.bit_length() - 1
        c = float(np.float64(c0) + 0.0)
        for l in range(depth):
            up = (k >> (depth - 1 - l)) & 1
            c = float(np.float64(c) + np.float64(qs[l] if up else -qs[l]))
        table[k] = ord_image(c) if depth < T else c
    return table


def digits_table(x, c0, e0, levels, T, table):
    """keys_kernel with a table: T levels of heap search, then the recursion from the level-T
    centre with the edge fractions of the deeper levels."""
    xo = ord_image(x + 0.0)
    kk = 1
    out = []
    for _ in range(T):
        up = xo > table[kk]
        out.append(1 if up else 0)
        kk = 2 * kk + (1 if up else 0)
    c = table[kk]
    qs = q_sequence(e0, levels)
    for l in range(T, levels):
        up = xo > ord_image(c)
        out.append(1 if up else 0)
        c = float(np.float64(c) + np.float64(qs[l] if up else -qs[l]))
    return out


def _roots(rng):
    roots = [(0.5, 1.0), (0.0, 2.0), (-0.0, 1.0), (1e-17, 3.0), (-3.7, 0.123456789), (1234.5678, 1e-6),
             (0.1, 0.30000000000000004), (0.7, 0.0)]
    for _ in range(12):
        roots.append((float(rng.normal() * 10.0 ** rng.uniform(-5, 5)), float(10.0 ** rng.uniform(-8, 8))))
    return roots


@pytest.mark.parametrize("T", [4, 6, 8])
def test_key_table_search_equals_recursion(T):
    rng = np.random.default_rng(T)
    levels = 14
    for c0, e0 in _roots(rng):
        table = build_table(c0, e0, T)
        xs = list(c0 + e0 * rng.uniform(-0.6, 0.6, 200))
        # coordinates on the centres of the first levels, signed zeros, far outside the box
        xs += [c for c in table[1:2 << T] if isinstance(c, float)][:40]
        xs += [c0, c0 + 0.0, -0.0, 0.0, c0 + 10.0 * e0 + 1.0, c0 - 10.0 * e0 - 1.0]
        for x in xs:
            a = digits_recursion(float(x), c0, e0, levels)
            b = digits_table(float(x), c0, e0, levels, T, table)
            assert a == b, (c0, e0, x, a, b)


def test_timestep_estimate_error_bound():
    rng = np.random.default_rng(5)
    n = 200000
    for dim in (1, 2, 3):
        # the largest component and h within [2^-60, 2^60]; smaller components of any size down to 0
        amax = 2.0 ** rng.uniform(-60, 60, n)
        acc = np.zeros((n, dim))
        acc[:, 0] = amax * rng.choice([-1.0, 1.0], n)
        for k in range(1, dim):
            acc[:, k] = amax * rng.uniform(-1, 1, n) * 10.0 ** rng.uniform(-40, 0, n)
        h = 2.0 ** rng.uniform(-60, 60, n)
        af = acc.astype(np.float32)
        a2 = np.zeros(n, dtype=np.float32)
        for k in range(dim):
            a2 = np.float32(a2 + af[:, k] * af[:, k])
        e = np.sqrt(np.float32(h.astype(np.float32) / np.sqrt(a2)))
        exact = np.sqrt(h.astype(np.longdouble) / np.sqrt((acc.astype(np.longdouble) ** 2).sum(axis=1)))
        rel = np.abs(e.astype(np.longdouble) / exact - 1)
        assert float(rel.max()) < 4 * 2.0 ** -24, float(rel.max())
