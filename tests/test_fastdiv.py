"""Division by multiplication as the step kernel does it for site coordinates
(FastDiv in kmc_device.cuh): q = (n * m) >> p with p = 32 + ceil(log2 d) and
m = ceil(2^p / d) equals n // d for every divisor d in [1, 2^28] and n < 2^31.  Checked
with exact integer arithmetic on random and boundary cases (the kernel's 64-bit product
cannot overflow there: n * m < 2^64)."""
import random


def fastdiv(d):
    l = 0
    while l < 31 and (1 << l) < d:
        l += 1
    p = 32 + l
    m = ((1 << p) + d - 1) // d
    return m, p


def test_fastdiv_exact():
    rnd = random.Random(7)
    divisors = list(range(1, 300)) + [1 << k for k in range(29)] + [(1 << k) + 1 for k in range(1, 28)] + \
        [(1 << k) - 1 for k in range(2, 29)] + [rnd.randrange(1, 1 << 28) for _ in range(2000)]
    for d in divisors:
        m, p = fastdiv(d)
        ns = [0, 1, d - 1, d, d + 1, (1 << 31) - 1, (1 << 31) - 2] + [rnd.randrange(0, 1 << 31) for _ in range(50)]
        ns += [k * d + e for k in (1, 2, 1000, ((1 << 31) - 1) // d) for e in (-1, 0, 1)]
        for n in ns:
            if 0 <= n < (1 << 31):
                assert n * m < (1 << 64)
                assert (n * m) >> p == n // d, (n, d)


def test_site_index_bit_arithmetic():
    """The step kernel forms idx = int(1 + ran_site * n) with (double)n and the
    truncation done on bit patterns; both equal the FP64 conversions for n in
    [1, 2^31) and ran_site in [0, 1)."""
    import numpy as np
    rnd = np.random.default_rng(3)
    ns = np.concatenate([np.arange(1, 5000), rnd.integers(1, 1 << 31, 20000), (1 << np.arange(31)),
                         (1 << np.arange(1, 31)) - 1]).astype(np.int64)
    rs = np.concatenate([rnd.random(ns.size - 3), [0.0, np.nextafter(1.0, 0), 0.5]])
    FRAC, IMPL = (1 << 52) - 1, 1 << 52
    for n, r in zip(ns.tolist(), rs.tolist()):
        e = n.bit_length() - 1
        dn = np.array([((1023 + e) << 52) | ((n << (52 - e)) & FRAC)], dtype=np.uint64).view(np.float64)[0]
        assert dn == float(n)
        q = np.float64(1.0) + np.float64(r) * dn
        qb = int(np.array([q]).view(np.int64)[0])
        qe = (qb >> 52) - 1023
        idx = ((qb & FRAC) | IMPL) >> (52 - qe)
        assert idx == int(q), (n, r)
