"""Seeded synthetic particle frames in the reference's ``.xyz`` model.

No public dataset ships with the reference (its ``main.cpp`` points at a
local directory of simulator output), so the workloads are generated:
jittered lattices with a constant rest density rho0 = 1000 and a particle
mass of rho0 * spacing^3, so that m / rho is the volume per particle.

Each generator returns a :class:`ParticleFrame` holding exactly what an
``.xyz`` file holds (FluidSurfaceReconstruction/data_format.txt:1-28):
bounding box, kernel radius, particle radius, particle mass, then
``x y z density`` per particle.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

RHO0 = 1000.0


@dataclass
class ParticleFrame:
    bbox_min: np.ndarray     # (3,) f32
    bbox_max: np.ndarray     # (3,) f32
    h: float                 # kernel radius
    particle_radius: float
    mass: float
    pos: np.ndarray          # (N,3) f32
    density: np.ndarray      # (N,) f32
    name: str = ""

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


def _lattice_block(counts, spacing, origin, rng, jitter):
    nx, ny, nz = counts
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    p = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    p = (p + 0.5) * spacing + np.asarray(origin, dtype=np.float64)
    if jitter > 0:
        p += rng.uniform(-jitter, jitter, size=p.shape)
    return p


def lattice_cube(n_side: int = 32, r: float = 0.0125, seed: int = 1, jitter_frac: float = 0.1,
                 origin=(0.0, 0.0, 0.0)) -> ParticleFrame:
    """Plain small workload: an n_side^3 lattice of spacing r in the corner of
    the unit box, each particle jittered uniformly by +-jitter_frac*r, h = 4r."""
    rng = np.random.default_rng(seed)
    p = _lattice_block((n_side, n_side, n_side), r, origin, rng, jitter_frac * r)
    n = p.shape[0]
    return ParticleFrame(
        bbox_min=np.zeros(3, np.float32), bbox_max=np.ones(3, np.float32), h=4.0 * r,
        particle_radius=r, mass=RHO0 * r ** 3, pos=p.astype(np.float32),
        density=np.full(n, RHO0, np.float32), name=f"lattice{n_side}^3 r={r}")


def lattice_count(n_particles: int, seed: int = 1, r_ref: float = 0.0125, n_ref: int = 32768,
                  jitter_frac: float = 0.1) -> ParticleFrame:
    """The lattice-cube generator rescaled to about n_particles: the block keeps
    the physical extent of a 32^3 block of spacing 0.0125 and the spacing
    shrinks with the particle count."""
    side = max(2, int(round(n_particles ** (1.0 / 3.0))))
    r = r_ref * (n_ref ** (1.0 / 3.0)) / side
    return lattice_cube(side, r, seed, jitter_frac)


def dam_break(n_total: int = 1 << 20, r: float = 0.004, seed: int = 2, splash_frac: float = 0.02,
              jitter_frac: float = 0.1) -> ParticleFrame:
    """Anisotropic workload: a 0.4 x 0.8 x 0.4 column at the box corner, a
    droplet of radius 0.08 centred at (0.7, 0.6, 0.5), and splash particles
    uniform in the top half of the unit box.  The lattice spacing s is chosen
    so that column + droplet hold about (1 - splash_frac) * n_total particles;
    the splash fills the count up to n_total exactly.  r is the particle
    radius and h = 4r."""
    rng = np.random.default_rng(seed)
    vol = 0.4 * 0.8 * 0.4 + 4.0 / 3.0 * math.pi * 0.08 ** 3
    target = (1.0 - splash_frac) * n_total
    s = (vol / target) ** (1.0 / 3.0)
    col = _lattice_block((int(round(0.4 / s)), int(round(0.8 / s)), int(round(0.4 / s))), s,
                         (0.0, 0.0, 0.0), rng, jitter_frac * r)
    m = int(math.ceil(0.16 / s)) + 1
    drop = _lattice_block((m, m, m), s, (0.7 - m * s / 2, 0.6 - m * s / 2, 0.5 - m * s / 2), rng,
                          jitter_frac * r)
    drop = drop[np.sum((drop - np.array([0.7, 0.6, 0.5])) ** 2, axis=1) <= 0.08 ** 2]
    body = np.concatenate([col, drop])
    if body.shape[0] > n_total:
        body = body[:n_total]
    n_splash = n_total - body.shape[0]
    splash = np.stack([rng.uniform(0.0, 1.0, n_splash), rng.uniform(0.5, 1.0, n_splash),
                       rng.uniform(0.0, 1.0, n_splash)], axis=1)
    p = np.concatenate([body, splash]).astype(np.float32)
    p = np.clip(p, 0.0, 1.0).astype(np.float32)
    n = p.shape[0]
    fr = ParticleFrame(bbox_min=np.zeros(3, np.float32), bbox_max=np.ones(3, np.float32), h=4.0 * r,
                       particle_radius=r, mass=RHO0 * s ** 3, pos=p,
                       density=np.full(n, RHO0, np.float32), name=f"dam-break N={n}")
    fr.lattice_spacing = s
    return fr


def sphere_ball(n_target: int = 262144, radius: float = 0.3, seed: int = 4, center=(0.5, 0.5, 0.5),
                jitter_frac: float = 0.1, displace_frac: float = 0.5) -> ParticleFrame:
    """Differentiation workload: a jittered lattice filling a sphere of the
    given radius with about n_target particles, then displaced by Gaussian
    noise of standard deviation displace_frac * r (r = lattice spacing)."""
    rng = np.random.default_rng(seed)
    s = (4.0 / 3.0 * math.pi * radius ** 3 / n_target) ** (1.0 / 3.0)
    m = int(math.ceil(2 * radius / s)) + 2
    c = np.asarray(center)
    p = _lattice_block((m, m, m), s, c - m * s / 2, rng, jitter_frac * s)
    p = p[np.sum((p - c) ** 2, axis=1) <= radius ** 2]
    p = p[:n_target]
    p = p + rng.normal(0.0, displace_frac * s, size=p.shape)
    n = p.shape[0]
    return ParticleFrame(bbox_min=np.zeros(3, np.float32), bbox_max=np.ones(3, np.float32), h=4.0 * s,
                         particle_radius=s, mass=RHO0 * s ** 3, pos=p.astype(np.float32),
                         density=np.full(n, RHO0, np.float32), name=f"sphere N={n}")


def format_example() -> ParticleFrame:
    """The 12-particle example of FluidSurfaceReconstruction/data_format.txt:17-28."""
    pos = np.array([
        [0.0199628, 0.02, 0.0199924], [0.0397894, 0.0199325, 0.02], [0.0598905, 0.02, 0.0199746],
        [0.0799356, 0.02, 0.0199719], [0.0999644, 0.02, 0.0199709], [0.119978, 0.02, 0.0199695],
        [0.139987, 0.02, 0.0199687], [0.159992, 0.02, 0.0199681], [0.179995, 0.02, 0.0199676],
        [0.199997, 0.02, 0.0199673], [0.219998, 0.02, 0.0199671], [0.239999, 0.02, 0.019967]],
        dtype=np.float32)
    dens = np.array([429.723, 577.938, 587.701, 591.818, 594.787, 596.445, 597.548, 598.255,
                     598.721, 599.019, 599.201, 599.297], dtype=np.float32)
    return ParticleFrame(bbox_min=np.array([-0.04, -0.04, -0.04], np.float32),
                         bbox_max=np.array([3.04, 2.04, 1.54], np.float32), h=0.036,
                         particle_radius=0.01, mass=0.00403914, pos=pos, density=dens,
                         name="data_format example")
