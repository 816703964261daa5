"""Seeded synthetic workloads of the batching and serving benchmarks.

Random numbers come from MT19937-64 (the generator of C++'s std::mt19937_64,
Matsumoto & Nishimura 2004) implemented here, so a seed gives the same
workload on every host and in any language that implements the generator.
Draw conventions (in this order, per item):

* real in [0, 1):            (next() >> 11) * 2**-53
* integer in [lo, hi]:       lo + floor(real * (hi - lo + 1))
* log-uniform in [a, b]:     exp(ln a + real * (ln b - ln a))
* exponential (rate r):      -ln(1 - real) / r
* weighted choice:           first index whose cumulative weight exceeds real * total

Lattice units throughout (dx = dt = 1).  The viscosity of a cavity with lid
velocity U, longest edge L and Reynolds number Re is nu = L * U / Re (the
reference's Reynolds definition, src/CLbmSolver.cpp:98 and :284), clamped so
that tau = 3 nu + 1/2 >= 0.51 (nu >= 1/300).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List

import numpy as np

MASK64 = (1 << 64) - 1


class MT19937_64:
    """The 64-bit Mersenne Twister (std::mt19937_64)."""

    N, M = 312, 156
    MATRIX_A = 0xB5026F5AA96619E9
    UPPER, LOWER = 0xFFFFFFFF80000000, 0x7FFFFFFF

    def __init__(self, seed: int = 5489):
        self.mt = [0] * self.N
        self.mt[0] = seed & MASK64
        for i in range(1, self.N):
            prev = self.mt[i - 1]
            self.mt[i] = (6364136223846793005 * (prev ^ (prev >> 62)) + i) & MASK64
        self.index = self.N

    def _twist(self):
        mt = self.mt
        for i in range(self.N):
            x = (mt[i] & self.UPPER) | (mt[(i + 1) % self.N] & self.LOWER)
            xa = x >> 1
            if x & 1:
                xa ^= self.MATRIX_A
            mt[i] = mt[(i + self.M) % self.N] ^ xa
        self.index = 0

    def next(self) -> int:
        if self.index >= self.N:
            self._twist()
        y = self.mt[self.index]
        self.index += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & MASK64

    def real(self) -> float:
        return (self.next() >> 11) * (1.0 / 9007199254740992.0)

    def integer(self, lo: int, hi: int) -> int:
        return lo + int(self.real() * (hi - lo + 1))

    def log_uniform(self, a: float, b: float) -> float:
        return math.exp(math.log(a) + self.real() * (math.log(b) - math.log(a)))

    def exponential(self, rate: float) -> float:
        return -math.log(1.0 - self.real()) / rate

    def choice(self, weights) -> int:
        total = float(sum(weights))
        x = self.real() * total
        acc = 0.0
        for i, w in enumerate(weights):
            acc += w
            if x < acc:
                return i
        return len(weights) - 1


NU_MIN = 1.0 / 300.0  # tau >= 0.51


def lattice_tau(nu: float, storage: str):
    """(tau, 1/tau) in the storage's arithmetic precision, tau = 0.5 (6 nu + 1)."""
    T = np.float64 if storage == "f64" else np.float32
    tau = T(0.5) * (T(6) * T(nu) + T(1))
    return float(tau), float(T(1) / tau)


@dataclass
class Cavity:
    size: tuple          # (nx, ny, nz) interior cells
    lid: float           # lid velocity (lattice units)
    reynolds: float      # requested Re
    nu: float            # lattice viscosity after the tau clamp
    steps: int = 0
    arrival: float = 0.0  # seconds after the start (serving)

    def solver_args(self, storage: str):
        _, inv_tau = lattice_tau(self.nu, storage)
        T = np.float64 if storage == "f64" else np.float32
        return self.size, inv_tau, float(T(self.lid))

    @property
    def cells(self) -> int:
        return int(self.size[0]) * int(self.size[1]) * int(self.size[2])


def viscosity(L: int, U: float, Re: float) -> float:
    return max(L * U / Re, NU_MIN)


def batch_workload(count: int = 512, seed: int = 0, edge=(16, 96), lid=(0.02, 0.1), re=(10.0, 2000.0),
                   steps: int = 2000) -> List[Cavity]:
    """Independent box cavities: each axis an independent integer in `edge`,
    lid velocity uniform in `lid`, Re log-uniform in `re`.  Draw order per
    cavity: nx, ny, nz, U, Re."""
    rng = MT19937_64(seed)
    out = []
    for _ in range(count):
        size = tuple(rng.integer(edge[0], edge[1]) for _ in range(3))
        U = lid[0] + rng.real() * (lid[1] - lid[0])
        Re = rng.log_uniform(re[0], re[1])
        out.append(Cavity(size=size, lid=U, reynolds=Re, nu=viscosity(max(size), U, Re), steps=steps))
    return out


SERVE_EDGES = (32, 48, 64, 96, 128, 192, 256)
SERVE_WEIGHTS = (0.25, 0.2, 0.2, 0.15, 0.1, 0.06, 0.04)


def serving_workload(count: int = 10000, seed: int = 1, rate: float = 200.0, steps=(500, 20000), lid: float = 0.05,
                     re=(10.0, 5000.0)) -> List[Cavity]:
    """Cube-cavity solve requests with Poisson arrivals.  Draw order per
    request: inter-arrival time, edge (weighted), steps, Re."""
    rng = MT19937_64(seed)
    t = 0.0
    out = []
    for _ in range(count):
        t += rng.exponential(rate)
        edge = SERVE_EDGES[rng.choice(SERVE_WEIGHTS)]
        n = rng.integer(steps[0], steps[1])
        Re = rng.log_uniform(re[0], re[1])
        out.append(Cavity(size=(edge, edge, edge), lid=lid, reynolds=Re, nu=viscosity(edge, lid, Re), steps=n,
                          arrival=t))
    return out
