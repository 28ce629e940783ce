"""Seeded synthetic puncture workloads.

batched_binaries(): the batched sweep of seeded binaries -- bare masses
U[0.3, 0.5], separations U[4, 12] along y, transverse momenta (along x,
opposite for the two holes) with |P| ~ U[0, 0.12], spins |S| <= 0.2 m^2 in
uniformly random directions, N from {33, 49, 65, 97}, 6..10 levels, 4th
order, Robin boundary.

served_binaries(): those binaries arriving as a Poisson stream.

served_stream(): the served request stream -- 1..4 punctures at positions
U[-10, 10]^3 with a minimum separation of 2 (rejection sampling), bare masses
U[0.2, 0.6], |P| <= 0.2, |S| <= 0.3 m^2, N from the allowed sizes in
[33, 129], order in {2, 4, 6, 8}, 6..10 levels; 10% add the scalar-field
source (ps_case 2, amplitude U[0, 0.05], radius U[5, 20], width w U[1, 3]
passed as sigma = w^2), with Poisson arrival times at a given rate.

The reference publishes no data set for this path: these are synthetic
inputs with the stated distributions.  Domain length L = 1000 (the reference's
pars/Punctures/TestBH.run) unless given.
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np

from . import Problem

ALLOWED_N = [33, 37, 41, 45, 49, 53, 57, 65, 73, 81, 89, 97, 105, 113, 129]


def _random_direction(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def batched_binaries(count: int = 256, seed: int = 1004, L: float = 1000.0,
                     sizes=(33, 49, 65, 97), levels=(6, 10)) -> List[Problem]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m = rng.uniform(0.3, 0.5, 2)
        sep = rng.uniform(4.0, 12.0)
        pmag = rng.uniform(0.0, 0.12)
        spins = [rng.uniform(0.0, 0.2) * mi * mi * _random_direction(rng) for mi in m]
        P = Problem(equation="Punctures")
        P.mp = [float(m[0]), float(m[1])]
        P.x, P.z = [0.0, 0.0], [0.0, 0.0]
        P.y = [sep / 2, -sep / 2]
        P.px, P.py, P.pz = [-pmag, pmag], [0.0, 0.0], [0.0, 0.0]
        P.sx = [float(s[0]) for s in spins]
        P.sy = [float(s[1]) for s in spins]
        P.sz = [float(s[2]) for s in spins]
        P.n = int(rng.choice(sizes))
        P.levels = int(rng.integers(levels[0], levels[1] + 1))
        P.order, P.L, P.nu1, P.nu2, P.tol = 4, L, 3, 20, 1e-10
        out.append(P)
    return out


def served_binaries(count: int, rate_hz: float, seed: int = 1006) -> List[Tuple[float, Problem]]:
    """The batched workload's binaries (batched_binaries, in order) arriving
    as a Poisson stream: (arrival time in s, problem) pairs with exponential
    inter-arrival times of mean 1 / rate_hz."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for P in batched_binaries(count):
        t += rng.exponential(1.0 / rate_hz)
        out.append((t, P))
    return out


def served_stream(count: int, rate_hz: float, seed: int = 1005, L: float = 1000.0,
                  sizes=None, orders=(2, 4, 6, 8), levels=(6, 10)) -> List[Tuple[float, Problem]]:
    """(arrival time in s, problem) pairs with exponential inter-arrival times."""
    rng = np.random.default_rng(seed)
    sizes = list(sizes or ALLOWED_N)
    t = 0.0
    out = []
    for _ in range(count):
        t += rng.exponential(1.0 / rate_hz)
        nbh = int(rng.integers(1, 5))
        pos = []
        while len(pos) < nbh:
            p = rng.uniform(-10.0, 10.0, 3)
            if all(np.linalg.norm(p - q) >= 2.0 for q in pos):
                pos.append(p)
        m = rng.uniform(0.2, 0.6, nbh)
        P = Problem(equation="Punctures")
        P.mp = [float(x) for x in m]
        P.x = [float(p[0]) for p in pos]
        P.y = [float(p[1]) for p in pos]
        P.z = [float(p[2]) for p in pos]
        mom = [rng.uniform(0.0, 0.2) * _random_direction(rng) for _ in range(nbh)]
        spin = [rng.uniform(0.0, 0.3) * mi * mi * _random_direction(rng) for mi in m]
        P.px, P.py, P.pz = ([float(v[a]) for v in mom] for a in range(3))
        P.sx, P.sy, P.sz = ([float(v[a]) for v in spin] for a in range(3))
        P.n = int(rng.choice(sizes))
        P.order = int(rng.choice(orders))
        P.levels = int(rng.integers(levels[0], levels[1] + 1))
        P.L, P.nu1, P.nu2, P.tol = L, 3, 20, 1e-10
        if rng.uniform() < 0.1:
            P.equation = "Punctures_scalar_field"
            P.ps_case = 2
            P.ps_phi0 = float(rng.uniform(0.0, 0.05))
            P.ps_r0 = float(rng.uniform(5.0, 20.0))
            w = float(rng.uniform(1.0, 3.0))
            P.ps_sigma = w * w
        out.append((t, P))
    return out
