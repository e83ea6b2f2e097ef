"""Seeded synthetic series for the benchmark and the tests.

There is no public dataset for these workloads; seeded generators stand in:
  logistic : x <- r*x*(1-x), r = 3.9, x0 ~ U(0.1, 0.9), 1000 transients
  lorenz   : x-component of the Lorenz system (sigma 10, rho 28, beta 8/3),
             RK4 with dt = 0.01, initial state ~ N(0, 1), 5000 transients,
             z-scored
  white    : Gaussian white noise N(0, 1)
  ar1      : AR(1) with phi = 0.95 and unit Gaussian innovations
All are generated in float64 and cast by the caller.
"""
from __future__ import annotations

import numpy as np


def logistic(n: int, seed: int, r: float = 3.9, transient: int = 1000) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = float(rng.uniform(0.1, 0.9))
    for _ in range(transient):
        v = r * v * (1.0 - v)
    out = np.empty(n)
    for i in range(n):
        v = r * v * (1.0 - v)
        out[i] = v
    return out


def lorenz_x(n: int, seed: int, dt: float = 0.01, transient: int = 5000,
             sigma: float = 10.0, rho: float = 28.0, beta: float = 8.0 / 3.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x, y, z = (float(v) for v in rng.standard_normal(3))

    def f(x, y, z):
        return sigma * (y - x), x * (rho - z) - y, x * y - beta * z

    out = np.empty(n)
    h2, h6 = dt / 2.0, dt / 6.0
    for i in range(transient + n):
        k1 = f(x, y, z)
        k2 = f(x + h2 * k1[0], y + h2 * k1[1], z + h2 * k1[2])
        k3 = f(x + h2 * k2[0], y + h2 * k2[1], z + h2 * k2[2])
        k4 = f(x + dt * k3[0], y + dt * k3[1], z + dt * k3[2])
        x += h6 * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0])
        y += h6 * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1])
        z += h6 * (k1[2] + 2 * k2[2] + 2 * k3[2] + k4[2])
        if i >= transient:
            out[i - transient] = x
    return (out - out.mean()) / out.std()


def white(n: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal(n)


def uneven_batch(count: int = 512, seed: int = 4, n_lo: int = 1000, n_hi: int = 64000,
                 nthr: int = 8):
    """The uneven batched workload: `count` series with lengths log-uniform in
    [n_lo, n_hi], each a seeded mix (random convex weights) of z-scored
    logistic-map, Lorenz-x and AR(1) series, float32; per series a random
    tau in 1..4, emb in 2..8, norm Euclidean or maximal, and `nthr`
    thresholds linearly spaced over 0.1..1.0 of the series' std."""
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        s = int(rng.integers(1 << 30))
        parts = [logistic(n, s), lorenz_x(n, s + 1, transient=1000), ar1(n, s + 2)]
        w = rng.dirichlet([1.0, 1.0, 1.0])
        x = sum(wk * (p - p.mean()) / p.std() for wk, p in zip(w, parts))
        x = x.astype(np.float32)
        sd = float(np.std(x.astype(np.float64)))
        jobs.append(dict(x=x, tau=int(rng.integers(1, 5)), emb=int(rng.integers(2, 9)),
                         norm=int(rng.integers(1, 3)),
                         thresholds=(np.linspace(0.1, 1.0, nthr) * sd).astype(np.float32),
                         lmin=2, vmin=2, calc_entr=1))
    return jobs


def ar1(n: int, seed: int, phi: float = 0.95) -> np.ndarray:
    e = np.random.default_rng(seed).standard_normal(n)
    out = np.empty(n)
    acc = 0.0
    for i in range(n):
        acc = phi * acc + e[i]
        out[i] = acc
    return out
