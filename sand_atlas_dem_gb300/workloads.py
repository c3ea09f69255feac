"""Seeded specimens for tests and the benchmark (host side).

* :func:`contact_lattice` — grains on a cubic lattice slightly tighter than
  their equivalent diameter, so neighbours overlap shallowly: a small,
  contact-rich specimen for parity checks.
* :func:`lattice_assembly` — the reference's dilute starting lattice
  (``src/sand_atlas_dem/simulation.py:26-56``) with per-grain lognormal scales.
* :func:`compress` — isotropic cell compression with drag on the GB300 engine
  until a target solid fraction, the preparation of the dense packings.
"""

import math

import numpy as np


def equivalent_diameter(shape):
    return (6 * shape.volume / math.pi) ** (1 / 3)


def random_rotations(n, seed):
    """Unit quaternions as ``simulation.py:75-78`` draws them."""
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    return q.astype(np.float32)


def contact_lattice(library, side, *, spacing=0.985, seed=3, scale_sigma=0.05, speed=0.0):
    """``side**3`` grains at ``spacing`` equivalent diameters, jittered."""
    rng = np.random.default_rng(seed)
    n = side**3
    l0 = float(np.median([equivalent_diameter(s) for s in library.shapes]))
    step = spacing * l0
    idx = np.stack(np.meshgrid(*([np.arange(side)] * 3), indexing="ij"), -1).reshape(-1, 3)
    positions = (idx + 0.5) * step + rng.normal(0, 0.01 * l0, (n, 3))
    cell = np.full(3, side * step)
    ids = rng.integers(0, len(library.shapes), n).astype(np.uint32)
    scales = np.exp(rng.normal(0, scale_sigma, n))
    rotations = random_rotations(n, seed + 1)
    velocities = rng.normal(0, speed, (n, 3)) if speed else np.zeros((n, 3))
    return dict(positions=positions, cell=cell, ids=ids, scales=scales, rotations=rotations,
                velocities=velocities)


def lattice_assembly(library, n, solid_fraction, *, seed=42, scale_median=1.0, scale_sigma=0.2):
    """Dilute lattice start (``simulation.py:26-56``) with lognormal grain scales."""
    rng = np.random.default_rng(seed)
    ids = rng.integers(len(library.shapes), size=n, dtype=np.uint32)
    scales = scale_median * np.exp(rng.normal(0.0, scale_sigma, n))
    radius = max(s.radius for s in library.shapes) * scales.max()
    side = int(np.ceil(n ** (1 / 3)))
    volume = sum(library.shapes[int(i)].volume * s**3 for i, s in zip(ids, scales))
    length = (volume / solid_fraction) ** (1 / 3)
    cell = np.full(3, length)
    spacing = cell / side
    if np.any(spacing <= 2.1 * radius):
        raise ValueError("Requested dilute assembly does not fit nonoverlapping bounding spheres")
    indices = np.stack(np.meshgrid(*([np.arange(side)] * 3), indexing="ij"), -1).reshape(-1, 3)
    indices = indices[rng.permutation(len(indices))[:n]]
    positions = (indices + 0.5) * spacing
    jitter = np.maximum(0, spacing - 2.1 * radius) * 0.1
    positions += rng.uniform(-1, 1, (n, 3)) * jitter
    return positions, cell, ids, scales


def solid_fraction(engine):
    volume = sum(engine.library.shapes[int(i)].volume * s**3 for i, s in zip(engine.ids, engine.scales))
    cell = engine.read("cell", np.float32, (3, 4))[0, :3].astype(float) * engine.length_unit
    return volume / float(np.prod(cell))


def compress(engine, target, *, rate, drag, chunk=50, max_steps=2_000_000, log=None):
    """Shrink the periodic cell at ``-rate`` (1/s per axis) until ``target``."""
    steps = 0
    while solid_fraction(engine) < target and steps < max_steps:
        phi = solid_fraction(engine)
        # Final approach: slow down so the last chunk lands near the target.
        remaining = math.log(target / phi) / 3
        r = min(rate, remaining / (chunk * engine.spec.timestep) + 1e-9)
        engine.advance(chunk, rate=(-r, -r, -r), drag=drag)
        steps += chunk
        if log:
            log(steps, solid_fraction(engine))
    return steps
