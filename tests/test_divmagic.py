"""The invariant-divisor division the kernels use to turn a cell index into grid positions
(divmagic / divq in csrc/mol_device.cuh; Granlund and Montgomery, PLDI 1994, Fig. 4.1 with
N = 32): for every divisor up to 4096 and the grid sizes of the configurations, quotients of
indices up to 2^31 - 1 equal integer division, at random indices and at every multiple's
neighbours.  The GPU tests exercise the device code at every cell of every grid they run."""
import numpy as np


def divmagic(d):
    s = 0
    while s < 32 and (1 << s) < d:
        s += 1
    return ((((1 << s) - d) << 32) // d + 1) & 0xFFFFFFFF, s


def divq(n, m, l):
    return (((m * n) >> 32) + n) >> l


def test_division_by_invariant_divisors():
    rng = np.random.default_rng(0)
    divisors = list(range(1, 4097)) + [65536, 65537, 257 * 256, 510, 1024 * 1024, 16777216, (1 << 31) - 1]
    for d in divisors:
        m, l = divmagic(d)
        assert 0 <= m < (1 << 32)
        ns = [int(x) for x in rng.integers(0, 1 << 31, size=64)] + [0, 1, (1 << 31) - 1]
        for k in (1, 2, 3, ((1 << 31) - 1) // d):
            ns += [k * d - 1, k * d, k * d + 1]
        for n in ns:
            if 0 <= n < (1 << 31):
                assert divq(n, m, l) == n // d, (d, n)
