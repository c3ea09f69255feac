"""Seeded specimens for tests and the benchmark (host side).

* :func:`contact_lattice` — grains on a cubic lattice slightly tighter than
  their equivalent diameter, so neighbours overlap shallowly: a small,
  contact-rich specimen for parity checks.
* :func:`lattice_assembly` — the reference's dilute starting lattice
  (``src/sand_atlas_dem/simulation.py:26-56``) with per-grain lognormal scales.
* :func:`compress` — isotropic cell compression with drag on the GB300 engine
  until a target solid fraction, the preparation of the dense packings.
"""

import json
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


def dilute_lattice(library, n, *, seed=42, scale_sigma=0.2, gap=2.2):
    """Densest cubic lattice whose spacing clears ``gap`` times the largest
    bounding radius (the non-overlap rule of ``simulation.py:43-47``)."""
    rng = np.random.default_rng(seed)
    ids = rng.integers(len(library.shapes), size=n, dtype=np.uint32)
    scales = np.exp(rng.normal(0.0, scale_sigma, n))
    radius = max(library.shapes[int(i)].radius * s for i, s in zip(ids, scales))
    side = int(np.ceil(n ** (1 / 3)))
    spacing = gap * radius
    indices = np.stack(np.meshgrid(*([np.arange(side)] * 3), indexing="ij"), -1).reshape(-1, 3)
    indices = indices[rng.permutation(len(indices))[:n]]
    positions = (indices + 0.5) * spacing
    return positions, np.full(3, side * spacing), ids, scales


def material_spec(library, ids, scales, *, friction=0.5, damping_ratio=0.3, policy="conservative",
                  timestep=None, **overrides):
    """Benchmark material: rho 2650, kn 1e12 Pa/m, kt 5e11, mu, and a normal
    traction viscosity cn = 2 zeta sqrt(kn m / A) for the median grain
    (mass and surface area of the grain of median equivalent diameter).
    The timestep defaults to one ulp below the conservative bound."""
    from .model import conservative_timestep
    from .spec import Experiment

    ids = np.asarray(ids)
    scales = np.asarray(scales, float)
    diameters = np.array([equivalent_diameter(library.shapes[int(i)]) * s for i, s in zip(ids, scales)])
    k = int(np.argsort(diameters)[len(diameters) // 2])
    shape, s = library.shapes[int(ids[k])], scales[k]
    mass = 2650.0 * shape.volume * s**3
    area = shape.areas.sum() * s**2
    cn = 2 * damping_ratio * math.sqrt(1e12 * mass / area)
    fields = dict(
        particles=len(ids), contact_geometry="mesh", density=2650.0, normal_stiffness=1e12,
        tangential_stiffness=5e11, friction=friction, normal_viscosity=cn, timestep_policy=policy,
        timestep=1e-12, max_overlap_fraction=0.01,
    )
    fields.update(overrides)
    spec = Experiment(**fields)
    if timestep is None:
        from dataclasses import replace

        limit = conservative_timestep(library, spec, ids, scales)
        spec = replace(spec, timestep=float(np.nextafter(limit, 0.0)))
    else:
        from dataclasses import replace

        spec = replace(spec, timestep=float(timestep))
    return spec


def dense_packing(library, n, target, *, seed=42, scale_sigma=0.2, speedup=3.0, rate=2000.0,
                  max_steps=600_000, chunk=500, log=None, device=None, checkpoint=None):
    """Seeded dense periodic packing prepared by GPU compression.

    Starts from :func:`dilute_lattice` with random orientations.  Phase 1
    shrinks the periodic cell under frictionless contacts, the active-contact
    timestep guard at ``speedup`` times the run timestep and a temporary 8%
    overlap tolerance, adapting the rate to keep the deepest overlap near 3%
    (a node-sampled surface is soft until several nodes engage, so collisions
    penetrate a few percent).  Phase 2 holds the volume with drag until the
    deepest overlap is below 0.5% of a diameter: the frictionless packing is
    below its jamming density, so overlaps relax.  Rejected chunks roll back
    and slow down.  Each phase is bounded by ``max_steps``; ``checkpoint``
    (a callable) receives the engine after every 100 chunks.
    """
    from dataclasses import replace

    from .engine import Engine
    from .model import RejectedStep

    positions, cell, ids, scales = dilute_lattice(library, n, seed=seed, scale_sigma=scale_sigma)
    run = material_spec(library, ids, scales)
    dt = run.timestep * speedup
    prep = replace(run, friction=0.0, timestep_policy="active-contact", timestep=dt,
                   max_overlap_fraction=0.08)
    e = Engine(library, prep, positions, cell, ids, scales, device=device)
    e.buffers["rotation"].copy_from_numpy(random_rotations(n, seed + 1))
    e.initialize()
    history = []

    def report(phase, steps, r, overlap, rejected):
        row = dict(phase=phase, steps=steps, phi=round(solid_fraction(e), 4), rate=round(r, 2),
                   overlap=round(float(overlap), 5), rejected=rejected)
        history.append(row)
        if log and steps % (20 * chunk) == 0:
            log(row)
        if checkpoint and steps % (100 * chunk) == 0:
            checkpoint(e)

    r, steps, rejected = rate, 0, 0
    while solid_fraction(e) < target:
        if steps >= max_steps:
            raise RuntimeError(f"compression did not reach solid fraction {target} in {max_steps} steps")
        room = math.log(target / solid_fraction(e)) / 3 / (chunk * dt)
        step_rate = min(r, room + 1e-6)
        try:
            e.advance(chunk, rate=(-step_rate,) * 3, drag=0.002 / dt)
        except RejectedStep as exc:
            if exc.flags & ~(4 | 8192):
                raise
            rejected += 1
            r = max(r * 0.5, 1.0)
            continue
        steps += chunk
        overlap = e.diagnostics()["max_overlap_fraction"]
        r = max(r * 0.8, 1.0) if overlap > 0.035 else min(r * 1.15, 2 * rate) if overlap < 0.025 else r
        report("compress", steps, r, overlap, rejected)
    relax = 0
    overlap = e.diagnostics()["max_overlap_fraction"]
    while overlap > 0.005:
        if relax >= max_steps:
            raise RuntimeError(f"overlaps did not relax below 0.5% in {max_steps} steps")
        e.advance(chunk, drag=0.01 / dt)
        relax += chunk
        overlap = e.diagnostics()["max_overlap_fraction"]
        report("relax", relax, 0.0, overlap, rejected)
    state = e.state()
    return dict(state=state, ids=ids, scales=scales, spec=run, steps=steps + relax,
                cell=state["cell"][0, :3].astype(float) * e.length_unit, length_unit=e.length_unit,
                history=history, engine=e)


def save_packing(path, engine, ids, scales, meta):
    """Compact packing record: float64 centres, float32 orientations, cell."""
    state = engine.state()
    l0 = engine.length_unit
    positions = (state["position"][:, :3].astype(float) + state["positionRemainder"][:, :3]) * l0
    np.savez_compressed(path, positions=positions, rotations=state["rotation"].astype(np.float32),
                        cell=state["cell"][0, :3].astype(float) * l0, ids=np.asarray(ids, np.uint32),
                        scales=np.asarray(scales, float), meta=np.array(json.dumps(meta)))


def load_packing(path):
    with np.load(path, allow_pickle=False) as z:
        return dict(positions=z["positions"], rotations=z["rotations"], cell=z["cell"], ids=z["ids"],
                    scales=z["scales"], meta=json.loads(str(z["meta"])))


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


def main(argv=None):
    """``python -m sand_atlas_dem_gb300.workloads prepare --grains N --out file.npz``."""
    import argparse
    import sys
    import time

    from .shapes import synthetic_library

    p = argparse.ArgumentParser(prog="sand_atlas_dem_gb300.workloads")
    p.add_argument("command", choices=("prepare",))
    p.add_argument("--grains", type=int, default=10_000)
    p.add_argument("--library", default="f8", choices=("f4", "f8", "uneven"))
    p.add_argument("--solid-fraction", type=float, default=0.58)
    p.add_argument("--seed", type=int, default=42)
    p.add_argument("--out", required=True)
    args = p.parse_args(argv)
    library = synthetic_library(args.library)
    start = time.perf_counter()
    meta = dict(library=args.library, grains=args.grains, solid_fraction=args.solid_fraction, seed=args.seed)

    def checkpoint(engine):
        save_packing(args.out + ".partial.npz", engine, engine.ids, engine.scales, dict(meta, partial=True))

    out = dense_packing(library, args.grains, args.solid_fraction, seed=args.seed,
                        log=lambda row: print(json.dumps(row), file=sys.stderr, flush=True),
                        checkpoint=checkpoint)
    meta.update(steps=out["steps"], seconds=round(time.perf_counter() - start, 1),
                achieved_solid_fraction=solid_fraction(out["engine"]),
                max_overlap_fraction=out["history"][-1]["overlap"] if out["history"] else 0.0)
    save_packing(args.out, out["engine"], out["ids"], out["scales"], meta)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
