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


def precision_signals(n, batch, seed, device="cuda"):
    """The precision workload: each signal a sum of 64 complex sinusoids of random frequency (uniform on
    [0, n), not on the bin grid), amplitude (uniform on [0, 1)) and phase, plus 1e-3 N(0,1) complex noise.
    Parameters come from a seeded numpy stream; the sum is evaluated in FP64 on `device` and rounded to c32
    once.  Returns a numpy complex64 array (batch, n)."""
    import torch

    rng = np.random.default_rng(seed)
    t = torch.arange(n, dtype=torch.float64, device=device) / n
    out = np.empty((batch, n), np.complex64)
    for b in range(batch):
        f, a, ph = rng.uniform(0, n, 64), rng.uniform(0, 1, 64), rng.uniform(0, 2 * np.pi, 64)
        x = torch.zeros(n, dtype=torch.complex128, device=device)
        for i in range(64):
            x += float(a[i]) * torch.exp(1j * (2 * math.pi * float(f[i]) * t + float(ph[i])))
        noise = rng.standard_normal((2, n))
        x += 1e-3 * torch.complex(torch.from_numpy(noise[0]), torch.from_numpy(noise[1])).to(device)
        out[b] = x.to(torch.complex64).cpu().numpy()
    return out
