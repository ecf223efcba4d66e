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


def spray_frame(n=6000, radius=0.02, seed=21, jitter=0.2) -> Frame:
    """A jittered lattice slab with spray above it: 3 % of the particles as
    singletons, pairs and triples (splash particles: <= 2 neighbours within
    4r) and 7 % as loose Gaussian droplets (sigma = 2r, 4-12 particles),
    whose edge particles may or may not have three neighbours."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * radius
    n_small = max(3, int(0.03 * n))
    n_drop = int(0.07 * n)
    n_slab = n - n_small - n_drop

    def slab(s):
        return _lattice_box((0.0, 0.0, 0.0), (0.6 * s, 0.1 * s, 0.6 * s), sp)

    pts, s = _scaled_lattice(slab, n_slab, rng)
    pts = _jitter(pts, jitter * radius, rng)
    parts = [pts]
    left = n_small
    while left > 0:
        k = int(min(left, rng.integers(1, 4)))
        ctr = np.array([rng.uniform(0, 0.6 * s), rng.uniform(0.2 * s, 0.6 * s), rng.uniform(0, 0.6 * s)])
        parts.append(ctr + rng.uniform(-1.5 * radius, 1.5 * radius, size=(k, 3)))
        left -= k
    left = n_drop
    while left > 0:
        k = int(min(left, rng.integers(4, 13)))
        ctr = np.array([rng.uniform(0, 0.6 * s), rng.uniform(0.2 * s, 0.6 * s), rng.uniform(0, 0.6 * s)])
        parts.append(ctr + rng.normal(0.0, 2.0 * radius, size=(k, 3)))
        left -= k
    return Frame(np.concatenate(parts), radius, s, seed, "spray_%d" % n)


CONFIGS = {
    "slab_sphere": slab_and_sphere,
    "dam_break": dam_break,
    "small_blob": small_blob,
}


def _sphere_or_slab(rng, n, radius, jitter, domain=1.0):
    """One jittered-lattice sphere (radius 0.05-0.3) or slab in the unit box."""
    sp = 2.0 * radius
    if rng.random() < 0.5:
        R = rng.uniform(0.05, 0.3)
        c = rng.uniform(R, domain - R, size=3)
        pts = _lattice_sphere(c, R, sp)
    else:
        ext = rng.uniform(0.1, 0.6, size=3)
        ext[rng.integers(3)] = rng.uniform(2 * sp, 0.1)  # one thin axis
        lo = rng.uniform(0.0, domain - ext)
        pts = _lattice_box(lo, lo + ext, sp)
    if len(pts) > n:
        pts = pts[np.sort(rng.choice(len(pts), n, replace=False))]
    return _jitter(pts, jitter * radius, rng)


def _sorted_unique(a):
    """np.unique of an int64 array (sorted distinct values) by a sort and a
    neighbour comparison, which is several times faster than numpy's
    hash-based unique on millions of lattice keys."""
    a = np.sort(a)
    if len(a) == 0:
        return a
    return a[np.concatenate([[True], a[1:] != a[:-1]])]


def mixed_frame(seed, n_target, radius=0.01, jitter=0.2) -> Frame:
    """Batched-form frame: a seeded union of 1-6 jittered-lattice spheres and
    slabs in a unit box.  The shapes are drawn first; the whole set is then
    scaled about the origin (the geometry rule) until it holds n_target
    particles, and a seeded subset of n_target is kept."""
    rng = np.random.default_rng(seed)
    k = int(rng.integers(1, 7))
    shapes = [(rng.random() < 0.5, rng.random(5), int(rng.integers(3))) for _ in range(k)]
    sp = 2.0 * radius

    def build(s):
        out = []
        for is_sphere, u, ax in shapes:
            if is_sphere:
                R = (0.05 + 0.25 * u[0]) * s
                c = (R / s + (1 - 2 * R / s) * u[1:4]) * s
                out.append(_lattice_sphere(c, R, sp))
            else:
                ext = (0.1 + 0.5 * u[:3]) * s
                ext[ax] = max(2 * sp, 0.1 * u[3] * s)
                lo = (1 * s - ext) * u[1:4] * 0.999
                out.append(_lattice_box(lo, lo + ext, sp))
        pts = np.concatenate(out) if out else np.zeros((0, 3))
        ijk = np.round(pts / sp).astype(np.int64)
        ijk -= ijk.min(0) if len(ijk) else 0
        m = int(ijk.max()) + 1 if len(ijk) else 1
        key = _sorted_unique((ijk[:, 0] * m + ijk[:, 1]) * m + ijk[:, 2])
        return np.stack([key // (m * m), (key // m) % m, key % m], -1) * sp + \
            (np.round(pts.min(0) / sp) * sp if len(pts) else 0.0)

    # the lattice count grows as s^3: a few proportional steps reach the target
    s = 1.0
    for _ in range(60):
        pts = build(s)
        if len(pts) >= n_target:
            break
        s *= max(1.002, (n_target / max(len(pts), 1)) ** (1.0 / 3.0) * 1.002)
    pts = pts[np.sort(rng.choice(len(pts), size=n_target, replace=False))]
    pts = _jitter(pts, jitter * radius, rng)
    return Frame(pts, radius, s, seed, "mixed_%d_%d" % (seed, n_target))


def batch_frames(count=64, seed=100, n_min=50_000, n_max=2_000_000, radius=0.01):
    """The batched workload: `count` frames, particle counts log-uniform in
    [n_min, n_max]."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=count)).astype(int)
    return [mixed_frame(seed + 1 + i, int(n), radius) for i, n in enumerate(ns)]


def batch_frame(k, count=64, seed=100, n_min=50_000, n_max=2_000_000, radius=0.01):
    """Frame k of batch_frames(count, seed, ...) without building the others."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=count)).astype(int)
    return mixed_frame(seed + 1 + k, int(ns[k]), radius)


def batch_sizes(count=64, seed=100, n_min=50_000, n_max=2_000_000):
    """Particle counts of batch_frames(count, seed, ...)."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=count)).astype(int)


def _bezier(rng, t, scale):
    P = rng.uniform(0.1, 0.9, size=(4, 3)) * scale
    b = ((1 - t) ** 3)[:, None] * P[0] + (3 * (1 - t) ** 2 * t)[:, None] * P[1] + \
        (3 * (1 - t) * t ** 2)[:, None] * P[2] + (t ** 3)[:, None] * P[3]
    return b


def sheets_and_filaments(n=500_000, radius=0.01, seed=4) -> Frame:
    """Precision stress: 50 % thin sheets one to two particles thick on random
    planes and saddles z = a (x^2 - y^2), a in [0.5, 3]; 50 % filaments along
    random cubic Bezier curves with a 1-3 particle cross-section.  Spacing 2r.
    Near-degenerate neighbour covariances and ill-conditioned QEFs follow."""
    rng = np.random.default_rng(seed)
    sp = 2.0 * radius
    n_sheet = n // 2
    n_fil = n - n_sheet
    scale = max(1.0, (n / 500_000) ** 0.5 * 2.0)
    pts = []
    # sheets: lattice patches of side L on planes or saddles
    left = n_sheet
    while left > 0:
        L = rng.uniform(0.2, 0.5) * scale
        m = int(L / sp)
        u = (np.arange(m) - m / 2) * sp
        uu, vv = np.meshgrid(u, u, indexing="ij")
        layers = int(rng.integers(1, 3))
        if rng.random() < 0.5:
            a = rng.uniform(0.5, 3.0) / scale
            ww = a * (uu ** 2 - vv ** 2)
        else:
            ww = np.zeros_like(uu)
        patch = []
        for l in range(layers):
            patch.append(np.stack([uu.ravel(), vv.ravel(), ww.ravel() + l * sp], -1))
        patch = np.concatenate(patch)
        Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        c = rng.uniform(0.3, 0.7, size=3) * scale
        patch = patch @ Q.T + c
        take = min(left, len(patch))
        pts.append(patch[:take])
        left -= take
    left = n_fil
    while left > 0:
        length = 2.0 * scale
        m = max(int(length / sp), 8)
        t = np.linspace(0, 1, m)
        line = _bezier(rng, t, scale)
        k = int(rng.integers(1, 4))
        offs = [np.zeros(3)] + [rng.normal(size=3) * sp for _ in range(k - 1)]
        fil = np.concatenate([line + o for o in offs])
        take = min(left, len(fil))
        pts.append(fil[:take])
        left -= take
    pts = np.concatenate(pts)
    pts = _jitter(pts, 0.1 * radius, rng)
    return Frame(pts, radius, scale, seed, "sheets_filaments_%d" % n)


@dataclasses.dataclass
class VarFrame(Frame):
    radii: np.ndarray = None  # (n,) float32 per-particle radii


def two_radius_frame(n=20000, seed=6, r_small=0.01, r_large=0.02, jitter=0.2) -> VarFrame:
    """Variable-radius frame: a jittered-lattice slab of small particles
    (radius r_small, spacing 2 r_small) under a jittered-lattice sphere of
    large particles (radius r_large, spacing 2 r_large), each half of the
    particles; the geometry is scaled about the origin until each part holds
    its count, as the other generators do."""
    rng = np.random.default_rng(seed)
    n_small = n // 2
    n_large = n - n_small
    slab = lambda s: _lattice_box(np.array([0.0, 0.0, 0.0]), np.array([0.6, 0.15, 0.6]) * s, 2 * r_small)
    pts_s, s1 = _scaled_lattice(slab, n_small, rng)
    sph = lambda s: _lattice_sphere(np.array([0.3, 0.45, 0.3]) * s1, 0.18 * s, 2 * r_large)
    pts_l, _ = _scaled_lattice(sph, n_large, rng)
    pts = np.concatenate([_jitter(pts_s, jitter * r_small, rng), _jitter(pts_l, jitter * r_large, rng)])
    radii = np.concatenate([np.full(len(pts_s), r_small, np.float32), np.full(len(pts_l), r_large, np.float32)])
    return VarFrame(pts, r_small, s1, seed, "two_radius_%d" % n, radii)


def advect(xyz, w, g, t, dt, steps=1, scale=1.0):
    """Swirl plus gravity u = (-w (y - 0.5), w (x - 0.5), -g t) in the unit box
    scaled by `scale` (the geometry rule scales the domain with the particle
    count), integrated `steps` explicit steps from time t and clamped to the
    box (serving workload sequences)."""
    p = xyz / scale
    for k in range(steps):
        tt = t + k * dt
        u = np.stack([-w * (p[:, 1] - 0.5), w * (p[:, 0] - 0.5), np.full(len(p), -g * tt)], -1)
        p = np.clip(p + dt * u, 0.0, 1.0)
    return p * scale


SERVE_G = 0.5     # gravity of the serving sequences (box units / time^2)
SERVE_DT = 0.002  # time step between frames of a sequence: 200 steps move
                  # particles by a few percent of the box instead of
                  # collapsing them onto the floor


def serving_requests(count=2000, seed=500, n_min=10_000, n_max=4_000_000, rate_hz=20.0):
    """Serving workload: `count` frame requests with Poisson arrivals at
    `rate_hz`, grouped into time-correlated sequences of 20-200 steps; each
    sequence has its own particle count (log-uniform), radius in
    {0.005, 0.01, 0.02} and swirl w in [0.5, 2].  Yields dicts with the
    arrival time and a callable that materialises the frame."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_hz, size=count))
    out = []
    i = 0
    seq = 0
    while i < count:
        length = int(rng.integers(20, 201))
        n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        r = float(rng.choice([0.005, 0.01, 0.02]))
        w = float(rng.uniform(0.5, 2.0))
        base_seed = seed * 1000 + seq
        for k in range(min(length, count - i)):
            out.append(dict(t=float(arrivals[i]), seq=seq, step=k, n=n, radius=r, w=w, seed=base_seed))
            i += 1
        seq += 1
    return out


def serving_frame(req, g=SERVE_G, dt=SERVE_DT) -> Frame:
    """Materialise one serving request: the sequence's base frame (a seeded
    mixed frame at spacing 2r in its scaled unit box) advected `step` steps."""
    fr = mixed_frame(req["seed"], req["n"], req["radius"])
    p = fr.xyz64
    if req["step"]:
        p = advect(p, req["w"], g, 0.0, dt, steps=req["step"], scale=fr.scale)
    return Frame(p, req["radius"], fr.scale, req["seed"], "serve_%d_%d" % (req["seq"], req["step"]))


CONFIGS.update({
    "batch64": batch_frames,
    "sheets_filaments": sheets_and_filaments,
    "serving": serving_requests,
})
