"""Seeded workloads of the batched and served forms.

Ensemble sampler: splitmix64 (Steele, Lea and Flood, "Fast splittable pseudorandom
number generators", 2014).  Run r draws from its own stream, whose state starts at
seed + r * 2^32; u = (x >> 11) * 2^-53 is a uniform double in [0, 1).  Per run:
  Nx  ~ U{1024..8192} rounded to a multiple of 32
  Np  ~ U{128..1024}  rounded to a multiple of 32
  a0  ~ U[0.5, 3]
  n   ~ logU[0.001, 0.05] n_c
  T   ~ U[0.1, 10] keV
  levels uniform in {1, 2}
with the rest of the laser / plasma-slab problem as in the single-run workloads.
Serving arrivals: a Poisson process (exponential inter-arrival times) from stream 0 of
its own seed.
"""
from __future__ import annotations

import math

MASK = (1 << 64) - 1
SEED_ENSEMBLE = 0x5EED0004
SEED_ARRIVALS = 0x5EED0005


class SplitMix64:
    def __init__(self, seed: int, stream: int = 0):
        self.state = (seed + (stream << 32)) & MASK

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next() >> 11) * (1.0 / (1 << 53))


def _round32(v: float, lo: int, hi: int) -> int:
    return int(min(hi, max(lo, 32 * round(v / 32))))


def ensemble_problems(count: int = 64, seed: int = SEED_ENSEMBLE, precision: int = 64):
    """The batched workload: `count` independent laser / slab problems."""
    from . import Problem

    out = []
    for r in range(count):
        g = SplitMix64(seed, r)
        nx = _round32(1024 + g.uniform() * (8192 - 1024), 1024, 8192)
        np_ = _round32(128 + g.uniform() * (1024 - 128), 128, 1024)
        a0 = 0.5 + 2.5 * g.uniform()
        dens = math.exp(math.log(0.001) + g.uniform() * (math.log(0.05) - math.log(0.001)))
        te = 0.1 + 9.9 * g.uniform()
        levels = 1 + int(g.uniform() * 2)
        out.append(Problem(L=100.0, nx=nx, np=np_, Lfinest=levels, r=2, pmax=2.0, dens=dens, x1=15, x2=20, x3=80,
                           x4=85, Te=te, a0=a0, fwhm=10.0, delay=10.0, cfl=0.5, quadDepth=2, crit=1e-6,
                           sizeWeight=1.0, precision=precision))
    return out


def arrival_times(count: int, rate: float = 20.0, seed: int = SEED_ARRIVALS) -> list[float]:
    """First `count` arrival times (seconds) of a Poisson process of the given rate."""
    g = SplitMix64(seed, 0)
    t, out = 0.0, []
    for _ in range(count):
        t += -math.log(1.0 - g.uniform()) / rate
        out.append(t)
    return out
