"""Seeded synthetic particle sets with the shapes of the five KDTree workloads.

The reference publishes no dataset for this path, so every workload is generated here
from a numpy PCG64 stream (``numpy.random.default_rng(seed)``):

* ``uniform_box``      -- 32768 particles uniform in the periodic unit box, m = 1/N.
* ``clustered_box``    -- 70% of the particles in 500 Plummer spheres (centres uniform,
  scale radius log-uniform in [0.05, 0.5], member counts drawn from dN/dn ~ n^-2 and
  rescaled to the 70% total, radii truncated at 10a), 30% uniform background, wrapped
  into [0, L). Optional Gaussian velocities: per sphere sigma^2 = (3 pi / 64) G M_s / a
  with G = 1 (the Plummer mass-weighted 1-D dispersion), sigma = 0.1 for the background.
* ``plummer_groups``   -- independent Plummer spheres (a = 1, Gaussian velocities with
  sigma = 1) whose sizes follow dN/dn ~ n^-2 on [20, 200000]; used by the batched path.
"""
from __future__ import annotations

import numpy as np


def _pareto_n2(rng, size, nmin, nmax):
    """Sizes with dN/dn proportional to n^-2 on [nmin, nmax] by inverse CDF."""
    u = rng.random(size)
    a, b = 1.0 / nmin, 1.0 / nmax
    return 1.0 / (a - u * (a - b))


def _plummer_radii(rng, count, a):
    """Plummer radii r = a / sqrt(u^(-2/3) - 1), redrawn until all lie below 10a."""
    r = np.empty(count)
    todo = np.arange(count)
    while todo.size:
        u = rng.random(todo.size)
        u = np.clip(u, 1e-300, 1.0 - 1e-16)
        rr = a[todo] / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        ok = rr < 10.0 * a[todo]
        r[todo[ok]] = rr[ok]
        todo = todo[~ok]
    return r


def _isotropic(rng, count):
    v = rng.normal(size=(count, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def uniform_box(n=32768, box=1.0, seed=1):
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 3)) * box
    mass = np.full(n, 1.0 / n)
    return pos, mass


def clustered_box(n=1 << 20, box=100.0, seed=2, nspheres=500, frac=0.7, velocities=False):
    rng = np.random.default_rng(seed)
    nclust = int(round(frac * n))
    raw = 1.0 / (1.0 - rng.random(nspheres))  # dN/dn ~ n^-2 for n >= 1
    counts = np.floor(raw / raw.sum() * nclust).astype(np.int64)
    counts[0] += nclust - counts.sum()
    centres = rng.random((nspheres, 3)) * box
    scale = np.exp(rng.uniform(np.log(0.05), np.log(0.5), nspheres))
    sphere = np.repeat(np.arange(nspheres), counts)
    a = scale[sphere]
    r = _plummer_radii(rng, nclust, a)
    pos_c = centres[sphere] + r[:, None] * _isotropic(rng, nclust)
    pos_b = rng.random((n - nclust, 3)) * box
    pos = np.mod(np.concatenate([pos_c, pos_b]), box)
    pos[pos >= box] = 0.0  # guard the rounding of mod at the upper wall
    mass = np.full(n, 1.0 / n)
    if not velocities:
        return pos, mass
    msph = counts * (1.0 / n)
    sig = np.sqrt(3.0 * np.pi / 64.0 * msph / scale)
    vel_c = rng.normal(size=(nclust, 3)) * sig[sphere][:, None]
    vel_b = rng.normal(size=(n - nclust, 3)) * 0.1
    vel = np.concatenate([vel_c, vel_b])
    return pos, mass, vel


def linking_length(n, box, b=0.2):
    """b times the mean interparticle spacing."""
    return b * box / n ** (1.0 / 3.0)


def group_sizes(ngroups=20000, nmin=20, nmax=200000, seed=4):
    rng = np.random.default_rng(seed)
    return np.floor(_pareto_n2(rng, ngroups, nmin, nmax)).astype(np.int64).clip(nmin, nmax)


def plummer_groups(sizes, seed=4, a=1.0, sigma=1.0):
    """Concatenated Plummer spheres; returns pos, vel, mass, offsets (CSR over groups)."""
    rng = np.random.default_rng(seed + 1000)
    sizes = np.asarray(sizes, np.int64)
    total = int(sizes.sum())
    aa = np.full(total, a)
    r = _plummer_radii(rng, total, aa)
    pos = r[:, None] * _isotropic(rng, total)
    vel = rng.normal(size=(total, 3)) * sigma
    mass = np.full(total, 1.0)
    offsets = np.zeros(sizes.size + 1, np.int64)
    np.cumsum(sizes, out=offsets[1:])
    return pos, vel, mass, offsets
