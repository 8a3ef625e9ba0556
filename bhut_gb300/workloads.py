"""Seeded synthetic N-body systems used by the tests and the benchmark.

There is no public dataset for this engine; every workload is generated from
a seed with numpy's PCG64 ``default_rng``:

* ``gaussian``: i.i.d. standard-normal positions, unit masses (the
  CPU-runnable 10,000-particle case).
* ``plummer``: Plummer sphere, r = a / sqrt(u^(-2/3) - 1) with radii beyond
  ``rmax * a`` redrawn, isotropic directions, equal masses 1/N.
  u^(1/3) is drawn as the largest of three uniforms (its CDF is v^3), so
  r = a v / sqrt(1 - v^2), and directions use Marsaglia's disc method: only
  correctly rounded IEEE operations are involved, so the same seed gives
  bit-identical systems on x86-64 and aarch64.
* ``uniform_cube``: uniform in a centred cube of the given side.
* ``galaxy``: 70 % exponential disc (radial scale ``rd`` drawn from
  Gamma(2, rd), sech^2 vertical profile z = z0 * atanh(2u - 1)) and 30 %
  Hernquist bulge (r = a sqrt(u) / (1 - sqrt(u)), radii beyond ``rmax * a``
  redrawn as for the Plummer sphere: untruncated, the sampler's tail puts a
  few particles at 1e6 a and inflates the box by orders of magnitude), equal
  masses 1/N.
"""
from __future__ import annotations

import numpy as np


def _isotropic(rng: np.random.Generator, n: int) -> np.ndarray:
    cos_t = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    sin_t = np.sqrt(np.maximum(0.0, 1.0 - cos_t * cos_t))
    return np.stack([sin_t * np.cos(phi), sin_t * np.sin(phi), cos_t], axis=1)


def gaussian(n: int, seed: int = 0, dim: int = 3):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n, dim)), np.ones(n)


def _marsaglia_directions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Isotropic unit vectors from points uniform in the unit disc."""
    out = np.empty((n, 3))
    todo = np.arange(n)
    while len(todo):
        x1 = rng.uniform(-1.0, 1.0, len(todo))
        x2 = rng.uniform(-1.0, 1.0, len(todo))
        s = x1 * x1 + x2 * x2
        ok = (s < 1.0) & (s > 0.0)
        idx = todo[ok]
        q = 2.0 * np.sqrt(1.0 - s[ok])
        out[idx, 0] = x1[ok] * q
        out[idx, 1] = x2[ok] * q
        out[idx, 2] = 1.0 - 2.0 * s[ok]
        todo = todo[~ok]
    return out


def plummer(n: int, seed: int = 0, a: float = 1.0, rmax: float = 20.0):
    rng = np.random.default_rng(seed)
    r = np.empty(n)
    todo = np.arange(n)
    while len(todo):
        k = len(todo)
        v = np.maximum(np.maximum(rng.uniform(0.0, 1.0, k), rng.uniform(0.0, 1.0, k)),
                       rng.uniform(0.0, 1.0, k))          # v = u^(1/3)
        ok = (v > 0.0) & (v < 1.0)
        rr = np.full(k, np.inf)
        rr[ok] = a * v[ok] / np.sqrt(1.0 - v[ok] * v[ok])
        ok &= rr <= rmax * a
        r[todo[ok]] = rr[ok]
        todo = todo[~ok]
    pos = _marsaglia_directions(rng, n) * r[:, None]
    return pos, np.full(n, 1.0 / n)


def uniform_cube(n: int, seed: int = 0, side: float = 10.0, dim: int = 3):
    rng = np.random.default_rng(seed)
    return rng.uniform(-side / 2, side / 2, (n, dim)), np.full(n, 1.0 / max(n, 1))


def galaxy(n: int, seed: int = 0, rd: float = 3.0, z0: float = 0.3, a_bulge: float = 0.5,
           disc_fraction: float = 0.7, rmax: float = 20.0):
    rng = np.random.default_rng(seed)
    nd = int(round(disc_fraction * n))
    nb = n - nd
    R = rng.gamma(2.0, rd, nd)
    phi = rng.uniform(0.0, 2.0 * np.pi, nd)
    u = rng.uniform(0.0, 1.0, nd)
    u = np.clip(u, 1e-15, 1.0 - 1e-15)
    z = z0 * np.arctanh(2.0 * u - 1.0)
    disc = np.stack([R * np.cos(phi), R * np.sin(phi), z], axis=1)
    rb = np.empty(nb)
    todo = np.arange(nb)
    while len(todo):
        s = np.sqrt(rng.uniform(0.0, 1.0, len(todo)))
        rr = a_bulge * s / np.maximum(1.0 - s, 1e-300)
        ok = rr <= rmax * a_bulge
        rb[todo[ok]] = rr[ok]
        todo = todo[~ok]
    bulge = _isotropic(rng, nb) * rb[:, None]
    pos = np.concatenate([disc, bulge], axis=0)
    return pos, np.full(n, 1.0 / n)


def plummer_batch(nsys: int = 2048, nmin: int = 256, nmax: int = 65536, seed: int = 0,
                  amin: float = 0.5, amax: float = 2.0):
    """Independent Plummer spheres: N log-uniform in [nmin, nmax], scale
    radius uniform in [amin, amax], each with its own seed, equal masses
    1/N.  Returns a list of (positions, masses)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), nsys)).astype(np.int64)
    scales = rng.uniform(amin, amax, nsys)
    seeds = rng.integers(0, 2**31 - 1, nsys)
    return [plummer(int(n), seed=int(sd), a=float(a)) for n, a, sd in zip(sizes, scales, seeds)]


def cube_targets(m: int, seed: int = 0, side: float = 10.0, dim: int = 3) -> np.ndarray:
    """External targets uniform in a centred cube of the given side."""
    rng = np.random.default_rng(seed)
    return rng.uniform(-side / 2, side / 2, (m, dim))
