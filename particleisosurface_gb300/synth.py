"""Seeded synthetic particle sets for the benchmark configurations.

The reference reconstructs SPH particle frames loaded from CSV/HDF5 case files
(src/main.cpp:215-328); none ship with it, so every frame here is synthetic
and reproducible from its seed.  Positions are generated in float64 and rounded
to float32, as the reference rounds its HDF5 doubles on load
(src/main.cpp:317-318).

Geometry rule.  The configurations state counts that do not fit their shapes
at lattice spacing 2r (a 0.6 x 0.2 x 0.6 slab holds about 720 points at
r = 0.025, not 16,000).  Counts, radius, spacing, jitter and proportions are
kept; every length of the configuration (shapes and domain) is scaled about the
origin by the smallest factor s (searched in 0.5 % steps from
(N_target / N_lattice)^(1/3)) at which the scaled lattice holds at least the
target count, and a seeded subset of exactly the target count is kept.  s is
returned with every frame.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Frame:
    xyz64: np.ndarray  # (n, 3) float64
    radius: float
    scale: float
    seed: int
    name: str

    @property
    def xyz(self) -> np.ndarray:
        return np.ascontiguousarray(self.xyz64.astype(np.float32))

    @property
    def n(self) -> int:
        return int(self.xyz64.shape[0])


def _lattice_box(lo, hi, spacing):
    axes = [np.arange(lo[k] + 0.5 * spacing, hi[k], spacing) for k in range(3)]
    g = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1).reshape(-1, 3)
    return g


def _lattice_sphere(c, rad, spacing):
    lo = np.asarray(c) - rad
    hi = np.asarray(c) + rad
    g = _lattice_box(lo, hi, spacing)
    return g[np.sum((g - np.asarray(c)) ** 2, axis=1) <= rad * rad]


def _scaled_lattice(make, n_target, rng):
    """make(s) -> lattice points for scale s; returns (points[n_target], s)."""
    n0 = max(len(make(1.0)), 1)
    s = max((n_target / n0) ** (1.0 / 3.0), 1e-3)
    for _ in range(2000):
        pts = make(s)
        if len(pts) >= n_target:
            sel = rng.choice(len(pts), size=n_target, replace=False)
            sel.sort()
            return pts[sel], s
        s *= 1.005
    raise RuntimeError("lattice scale search did not converge")


def _jitter(pts, amp, rng):
    return pts + rng.uniform(-amp, amp, size=pts.shape)


def slab_and_sphere(n=20000, radius=0.025, seed=1, jitter=0.2) -> Frame:
    """Plain single frame: 80 % on a 0.6 x 0.2 x 0.6 slab at y in [0, 0.2],
    20 % on a lattice inside a sphere of radius 0.12 at (0.3, 0.45, 0.3);
    spacing 2r, uniform jitter +-jitter*r."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * radius
    n_slab = int(round(0.8 * n))
    n_sph = n - n_slab

    def slab(s):
        return _lattice_box((0.0, 0.0, 0.0), (0.6 * s, 0.2 * s, 0.6 * s), sp)

    def sph(s):
        return _lattice_sphere((0.3 * s, 0.45 * s, 0.3 * s), 0.12 * s, sp)

    # One scale for the whole configuration: the larger of the two.
    _, s1 = _scaled_lattice(slab, n_slab, np.random.default_rng(seed))
    _, s2 = _scaled_lattice(sph, n_sph, np.random.default_rng(seed))
    s = max(s1, s2)
    a = slab(s)
    b = sph(s)
    a = a[np.sort(rng.choice(len(a), size=n_slab, replace=False))]
    b = b[np.sort(rng.choice(len(b), size=n_sph, replace=False))]
    pts = np.concatenate([a, b])
    pts = _jitter(pts, jitter * radius, rng)
    return Frame(pts, radius, s, seed, "slab_sphere_%d" % n)


def dam_break(n=1_000_000, radius=0.01, seed=2, jitter=0.25, spray_frac=0.15) -> Frame:
    """Plain GPU form at scale: 85 % fill a jittered 0.4 x 0.8 x 0.4 column
    (y up) at spacing 2r; 15 % are spray, Gaussian blobs (sigma = 3r) of 5-50
    particles with centres uniform above the column top inside the unit
    domain."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * radius
    n_col = int(round((1.0 - spray_frac) * n))
    n_spray = n - n_col

    def col(s):
        return _lattice_box((0.0, 0.0, 0.0), (0.4 * s, 0.8 * s, 0.4 * s), sp)

    _, s = _scaled_lattice(col, n_col, np.random.default_rng(seed))
    c = col(s)
    c = c[np.sort(rng.choice(len(c), size=n_col, replace=False))]
    c = _jitter(c, jitter * radius, rng)
    blobs = []
    left = n_spray
    while left > 0:
        k = int(min(left, rng.integers(5, 51)))
        ctr = np.array([rng.uniform(0, s), rng.uniform(0.8 * s, s), rng.uniform(0, s)])
        blobs.append(ctr + rng.normal(0.0, 3.0 * radius, size=(k, 3)))
        left -= k
    pts = np.concatenate([c] + blobs)
    return Frame(pts, radius, s, seed, "dam_break_%d" % n)


def small_blob(n=2000, radius=0.025, seed=3, jitter=0.2) -> Frame:
    """A small jittered lattice ball plus a few loose particles, for fast
    parity cases."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * radius
    n_loose = max(n // 50, 1)

    def ball(s):
        return _lattice_sphere((0.2 * s, 0.2 * s, 0.2 * s), 0.1 * s, sp)

    pts, s = _scaled_lattice(ball, n - n_loose, rng)
    pts = _jitter(pts, jitter * radius, rng)
    loose = rng.uniform(0.0, 0.4 * s, size=(n_loose, 3))
    return Frame(np.concatenate([pts, loose]), radius, s, seed, "small_blob_%d" % n)


CONFIGS = {
    "slab_sphere": slab_and_sphere,
    "dam_break": dam_break,
    "small_blob": small_blob,
}
