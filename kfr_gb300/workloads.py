"""Synthetic workloads with the shapes of the benchmark configurations (seeded; no dataset is involved)."""
import bisect
import math

import numpy as np


def _smooth_numbers(limit):
    out = []
    p2 = 1
    while p2 <= limit:
        p3 = p2
        while p3 <= limit:
            p5 = p3
            while p5 <= limit:
                p7 = p5
                while p7 <= limit:
                    out.append(p7)
                    p7 *= 7
                p5 *= 5
            p3 *= 3
        p2 *= 2
    return sorted(out)


def _primes(limit):
    sieve = np.ones(limit + 1, dtype=bool)
    sieve[:2] = False
    for i in range(2, int(limit ** 0.5) + 1):
        if sieve[i]:
            sieve[i * i::i] = False
    return np.nonzero(sieve)[0].tolist()


def uneven_lengths(count=8192, lo=64, hi=65536, prime_fraction=0.1, seed=20261206):
    """Lengths drawn log-uniform on [lo, hi], rounded (in log) to the nearest 2^a 3^b 5^c 7^d, with a
    `prime_fraction` of them replaced by the nearest prime."""
    rng = np.random.default_rng(seed)
    smooth = [s for s in _smooth_numbers(2 * hi) if s >= lo // 2]
    primes = _primes(2 * hi)
    logs = rng.uniform(math.log(lo), math.log(hi), count)
    forced = rng.random(count) < prime_fraction
    out = []
    for lg, pr in zip(logs, forced):
        v = math.exp(lg)
        table = primes if pr else smooth
        i = bisect.bisect_left(table, v)
        cands = [table[j] for j in (i - 1, i) if 0 <= j < len(table)]
        out.append(min(cands, key=lambda c: abs(math.log(c) - lg)))
    return out
