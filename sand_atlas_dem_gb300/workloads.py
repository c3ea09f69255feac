"""Seeded specimens for tests and the benchmark (host side).

* :func:`contact_lattice` — grains on a cubic lattice slightly tighter than
  their equivalent diameter, so neighbours overlap shallowly: a small,
  contact-rich specimen for parity checks.
* :func:`walled_lattice` — a jittered lattice in a nonperiodic domain boxed by six
  moving penalty planes (the wall-stage benchmark).
* :func:`lattice_assembly` — the reference's dilute starting lattice
  (``src/sand_atlas_dem/simulation.py:26-56``) with per-grain lognormal scales.
* :func:`compress` — isotropic cell compression with drag on the GB300 engine
  until a target solid fraction, the preparation of the dense packings.
"""

import json
import time
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


def lattice_at(library, side, solid_fraction, *, seed=3, scale_sigma=0.05):
    """``side**3`` grains on a jittered cubic lattice whose spacing gives
    ``solid_fraction`` (mean grain volume / spacing^3), random orientations.

    A contact-rich ordered stand-in for a dense random packing: every grain
    touches its lattice neighbours once the spacing is below one equivalent
    diameter (solid fractions above about 0.53 for these shapes)."""
    rng = np.random.default_rng(seed)
    n = side**3
    ids = rng.integers(0, len(library.shapes), n).astype(np.uint32)
    scales = np.exp(rng.normal(0, scale_sigma, n))
    mean_volume = float(np.mean([library.shapes[int(i)].volume * s**3 for i, s in zip(ids, scales)]))
    step = (mean_volume / solid_fraction) ** (1 / 3)
    l0 = float(np.median([equivalent_diameter(s) for s in library.shapes]))
    idx = np.stack(np.meshgrid(*([np.arange(side)] * 3), indexing="ij"), -1).reshape(-1, 3)
    positions = (idx + 0.5) * step + rng.normal(0, 0.01 * l0, (n, 3))
    return dict(positions=positions, cell=np.full(3, side * step), ids=ids, scales=scales,
                rotations=random_rotations(n, seed + 1))


def walled_lattice(library, side, solid_fraction, *, seed=5, press=0.02, strain_rate=0.5, friction=0.3):
    """``lattice_at`` grains in a nonperiodic domain one lattice step wider on
    every side, boxed by six penalty planes (xmin, xmax, ..., zmax) placed
    ``press`` median diameters inside the outer grains' nominal surfaces and
    moving inward at ``strain_rate`` (1/s) of the box half-width each.  The
    planes carry the grain material (kn 1e12, kt 5e11) and ``friction``."""
    from .boundaries import BOX_NORMALS

    case = lattice_at(library, side, solid_fraction, seed=seed)
    step = case["cell"][0] / side
    l0 = float(np.median([equivalent_diameter(s) for s in library.shapes]))
    positions = case["positions"] + step
    domain = case["cell"] + 2 * step
    low = step + 0.5 * step - 0.5 * l0 + press * l0
    high = step + (side - 0.5) * step + 0.5 * l0 - press * l0
    speed = strain_rate * 0.5 * (high - low)
    planes = [
        dict(normal=n.tolist(), offset=float(low if k % 2 == 0 else -high), velocity=(speed * n).tolist(),
             normal_stiffness=1e12, tangential_stiffness=5e11, friction=friction)
        for k, n in enumerate(BOX_NORMALS.astype(float))
    ]
    return dict(positions=positions, cell=domain, ids=case["ids"], scales=case["scales"],
                rotations=case["rotations"], planes=planes)


def specimen_set(library, count=128, *, seed=11, grains=(500, 4000), solid_fraction=(0.55, 0.60),
                 rate=(0.1, 1.0)):
    """Independent periodic specimens for one batched engine: grain counts
    uniform in ``grains`` (rounded to the nearest cube of a lattice side),
    solid fractions uniform in ``solid_fraction``, compression rates (1/s)
    uniform in ``rate``.  Returns the specimen tuples, their rotations and
    the per-specimen rates."""
    rng = np.random.default_rng(seed)
    specimens, rotations, rates = [], [], []
    for k in range(count):
        side = int(round(rng.uniform(*grains) ** (1 / 3)))
        case = lattice_at(library, side, rng.uniform(*solid_fraction), seed=seed + 1000 + k)
        specimens.append((case["positions"], case["cell"], case["ids"], case["scales"]))
        rotations.append(case["rotations"])
        rates.append(rng.uniform(*rate))
    return specimens, np.concatenate(rotations), np.asarray(rates)


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
                  max_steps=600_000, chunk=500, log=None, device=None, checkpoint=None, start=None):
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
    (a callable) receives the engine after every 100 chunks; ``start`` (a
    :func:`load_packing` record) resumes from a saved state.
    """
    from dataclasses import replace

    from .engine import Engine
    from .model import RejectedStep

    if start is None:
        positions, cell, ids, scales = dilute_lattice(library, n, seed=seed, scale_sigma=scale_sigma)
    else:
        positions, cell, ids, scales = start["positions"], start["cell"], start["ids"], start["scales"]
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


def _write(engine, name, array):
    buffer = engine.buffers[name]
    if isinstance(buffer, np.ndarray):
        buffer[...] = np.asarray(array, buffer.dtype).reshape(buffer.shape)
    else:
        buffer.copy_from_numpy(np.ascontiguousarray(array))


def _read(engine, name, dtype, shape):
    buffer = engine.buffers[name]
    if isinstance(buffer, np.ndarray):
        return buffer.reshape(-1).view(dtype)[: int(np.prod(shape))].reshape(shape).copy()
    return engine.read(name, dtype, shape)


def descent_packing(library, n, target, *, seed=42, scale_sigma=0.2, growth=1.003, overlap=0.05,
                    max_evaluations=40_000, max_inner=400, log=None, device=None, engine_cls=None, start=None,
                    max_seconds=None):
    """Seeded dense periodic packing by affine compression and force descent.

    Starts from :func:`dilute_lattice` with random orientations.  Each round
    shrinks the periodic cell (solid fraction x ``growth``, larger while the
    packing is loose; centres scaled affinely) and then relaxes the grains
    under their frictionless contact forces and torques of the exact
    mesh-surface law (the engine's own force pass at zero timestep) by FIRE
    on the centres with each grain's summed nodal contact stiffness as its
    mass, plus a Jacobi rotation step, moves capped at 0.3% of a diameter,
    until the deepest overlap is below ``overlap`` of a diameter.  The
    perturbed grains are rough and jam below 0.58 when overlaps must stay
    under 1%, so the dense benchmark packing uses a 5% tolerance (up to 8%
    when a round's relaxation stalls after ``max_inner`` iterations).

    ``start`` (a :func:`load_packing` record) resumes from a saved state.
    When ``max_evaluations`` (or ``max_seconds``) is spent before ``target`` the result has
    ``converged`` False and holds the state reached, for a later resume.
    """
    from dataclasses import replace

    if start is None:
        positions, cell, ids, scales = dilute_lattice(library, n, seed=seed, scale_sigma=scale_sigma)
    else:
        positions, cell, ids, scales = start["positions"], start["cell"], start["ids"], start["scales"]
    run = material_spec(library, ids, scales)
    prep = replace(run, friction=0.0, normal_viscosity=0.0, timestep_policy="active-contact",
                   max_overlap_fraction=0.5, contacts_per_particle=512)
    if engine_cls is None:
        from .engine import Engine

        e = Engine(library, prep, positions, cell, ids, scales, device=device)
    else:
        e = engine_cls(library, prep, positions, cell, ids, scales)
    l0 = e.length_unit
    x = np.asarray(positions, float) / l0
    box = np.asarray(cell, float) / l0
    volume = sum(library.shapes[int(i)].volume * s**3 for i, s in zip(ids, scales)) / l0**3
    config = e.config(dt=0, history=False)
    evaluations = 0

    def place():
        x[:] = x - np.floor(x / box) * box
        hi = x.astype(np.float32)
        lo = (x - hi.astype(float)).astype(np.float32)
        _write(e, "position", np.pad(hi, ((0, 0), (0, 1))))
        _write(e, "positionRemainder", np.pad(lo, ((0, 0), (0, 1))))
        rows = _read(e, "cell", np.float32, (3, 4))
        rows[0, :3] = box
        rows[2, :3] = box
        rows[1] = 0
        _write(e, "cell", rows)
        _write(e, "cellLog", np.zeros((2, 4), np.float32))
        ctrl = np.zeros(16, np.uint32)
        ctrl[4] = 1
        _write(e, "control", ctrl)

    def contacts_of():
        count = int(_read(e, "control", np.uint32, (16,))[2])
        side = e.sides[e.active]
        if isinstance(side["meta"], np.ndarray):
            return side["meta"][:count].copy(), side["normalArea"][:count].copy()
        return (e.m.read_prefix(side["meta"], 4 * count, np.uint32, shape=(count, 4)),
                e.m.read_prefix(side["normalArea"], 4 * count, np.float32, shape=(count, 4)))

    def forces():
        nonlocal evaluations
        place()
        e.forces(config, capture_kinematics=False)
        evaluations += 1
        f = _read(e, "force", np.float32, (n, 4))
        ctrl = _read(e, "control", np.uint32, (16,))
        if int(ctrl[0]) & ~4:
            from .model import RejectedStep

            raise RejectedStep(ctrl[0])
        meta, normal = contacts_of()
        half = 0.5 * normal[:, 3].astype(float)
        stiffness = (np.bincount(meta[:, 0].astype(np.int64), half, minlength=n)
                     + np.bincount(meta[:, 1].astype(np.int64), half, minlength=n))
        torque = _read(e, "torque", np.float32, (n, 4))[:, :3].astype(float)
        return f[:, :3].astype(float), float(f[:, 3].max()), int(ctrl[2]), stiffness, torque

    diameters = e.layout.body[:, 3].astype(float)
    radii = e.layout.body[:, 2].astype(float)
    cap = 0.003 * diameters
    relax = 0.4
    q = (random_rotations(n, seed + 1) if start is None else start["rotations"]).astype(float)
    _write(e, "rotation", q.astype(np.float32))

    def rotate(torque, stiffness):
        # Jacobi rotation step about the torque: stiffness x radius^2.
        angle = relax * torque / np.maximum(stiffness * radii**2, 1e-30)[:, None]
        norm = np.linalg.norm(angle, axis=1)
        angle *= np.minimum(1.0, 0.005 / np.maximum(norm, 1e-30))[:, None]
        w = np.concatenate([0.5 * angle, np.zeros((n, 1))], axis=1)
        # q' = q + 0.5 [angle, 0] (x) q, renormalized (world-frame spin).
        a, b = w, q
        prod = np.empty_like(q)
        prod[:, :3] = a[:, 3:4] * b[:, :3] + b[:, 3:4] * a[:, :3] + np.cross(a[:, :3], b[:, :3])
        prod[:, 3] = a[:, 3] * b[:, 3] - np.einsum("ij,ij->i", a[:, :3], b[:, :3])
        q[:] = q + prod
        q[:] = q / np.linalg.norm(q, axis=1)[:, None]
        _write(e, "rotation", q.astype(np.float32))
    history = []
    phi = volume / np.prod(box)
    # FIRE (Bitzek et al., PRL 97, 170201, 2006) on the centres, with each
    # grain's summed contact stiffness as its mass (unit natural frequency),
    # plus a Jacobi rotation step about the torque.
    velocity = np.zeros((n, 3))
    converged = True
    deadline = time.perf_counter() + max_seconds if max_seconds else None
    while True:
        force, worst, contacts, stiffness, torque = forces()
        inner = 0
        dt, alpha, positive = 0.2, 0.1, 0
        velocity[:] = 0
        while worst > overlap:
            if evaluations >= max_evaluations or (deadline and time.perf_counter() > deadline):
                converged = False
                break
            if inner >= max_inner and worst < 1.6 * overlap:
                break  # slow tail: accept and keep compressing
            mass = np.maximum(stiffness, 1e-3 * stiffness.max() if stiffness.max() > 0 else 1.0)
            power = float(np.sum(force * velocity))
            fnorm, vnorm = np.linalg.norm(force), np.linalg.norm(velocity)
            if power > 0:
                velocity = (1 - alpha) * velocity + alpha * vnorm * force / max(fnorm, 1e-30)
                positive += 1
                if positive > 5:
                    dt, alpha = min(dt * 1.1, 1.0), alpha * 0.99
            else:
                velocity[:] = 0
                dt, alpha, positive = dt * 0.5, 0.1, 0
            velocity += dt * force / mass[:, None]
            move = dt * velocity
            norm = np.linalg.norm(move, axis=1)
            move *= np.minimum(1.0, cap / np.maximum(norm, 1e-30))[:, None]
            x += move
            rotate(torque, stiffness)
            force, worst, contacts, stiffness, torque = forces()
            inner += 1
        history.append(dict(phi=round(float(phi), 4), overlap=round(worst, 5), contacts=contacts, inner=inner,
                            evaluations=evaluations))
        if log and len(history) % 20 == 0:
            log(history[-1])
        if phi >= target * (1 - 1e-9) or not converged:
            break
        # Larger increments while the packing is loose.
        step = 1.05 if contacts == 0 else 1.01 if worst < 0.25 * overlap else growth
        next_phi = min(target, phi * step)
        factor = (phi / next_phi) ** (1 / 3)
        x *= factor
        box *= factor
        phi = volume / np.prod(box)
    _write(e, "velocity", np.zeros((n, 4), np.float32))
    return dict(engine=e, ids=ids, scales=scales, history=history, evaluations=evaluations,
                phi=float(phi), overlap=worst, spec=run, converged=converged and worst <= 1.6 * overlap)


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


def tile_packing(record, reps=(2, 2, 2)):
    """A periodic packing repeated ``reps`` times along each axis: copies of
    every grain (same shape, scale and orientation) shifted by whole cells,
    in a cell ``reps`` times larger.  The result is a periodic packing of the
    same solid fraction and the same contacts per grain, ``prod(reps)`` times
    larger (grain k of copy (a, b, c) is grain ``k + n (a reps[1] reps[2] +
    b reps[2] + c)``)."""
    positions = np.asarray(record["positions"], float)
    cell = np.asarray(record["cell"], float)
    shifts = np.stack(np.meshgrid(*(np.arange(r) for r in reps), indexing="ij"), -1).reshape(-1, 3)
    tiled = (positions[None, :, :] + (shifts * cell)[:, None, :]).reshape(-1, 3)
    copies = len(shifts)
    return dict(positions=tiled, cell=cell * np.asarray(reps, float),
                rotations=np.tile(np.asarray(record["rotations"]), (copies, 1)),
                ids=np.tile(np.asarray(record["ids"], np.uint32), copies),
                scales=np.tile(np.asarray(record["scales"], float), copies), meta=dict(record.get("meta", {})))


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

    from .shapes import synthetic_library

    p = argparse.ArgumentParser(prog="sand_atlas_dem_gb300.workloads")
    p.add_argument("command", choices=("prepare",))
    p.add_argument("--grains", type=int, default=10_000)
    p.add_argument("--library", default="f8", choices=("f4", "f8", "uneven"))
    p.add_argument("--solid-fraction", type=float, default=0.58)
    p.add_argument("--seed", type=int, default=42)
    p.add_argument("--out", required=True)
    p.add_argument("--resume", help="continue from a saved (partial) packing record")
    p.add_argument("--max-evaluations", type=int, default=40_000)
    p.add_argument("--max-seconds", type=float, default=None)
    p.add_argument("--overlap", type=float, default=0.05,
                   help="deepest overlap (fraction of a diameter) each relaxation must reach")
    args = p.parse_args(argv)
    library = synthetic_library(args.library)
    start = time.perf_counter()
    meta = dict(library=args.library, grains=args.grains, solid_fraction=args.solid_fraction, seed=args.seed)

    resume = load_packing(args.resume) if args.resume else None
    before = resume["meta"] if resume else {}
    out = descent_packing(library, args.grains, args.solid_fraction, seed=args.seed, start=resume,
                          overlap=args.overlap, max_evaluations=args.max_evaluations, max_seconds=args.max_seconds,
                          log=lambda row: print(json.dumps(row), file=sys.stderr, flush=True))
    meta.update(method="affine compression with frictionless force descent",
                evaluations=out["evaluations"] + before.get("evaluations", 0),
                seconds=round(time.perf_counter() - start + before.get("seconds", 0), 1),
                achieved_solid_fraction=out["phi"], max_overlap_fraction=out["overlap"])
    path = args.out if out["converged"] else args.out + ".partial.npz"
    save_packing(path, out["engine"], out["ids"], out["scales"], meta)
    print(json.dumps(dict(meta, converged=out["converged"], saved=path)))
    if not out["converged"]:
        sys.exit(3)


if __name__ == "__main__":
    main()


def packing_library(shapes=53, distinct=8, frequency=40, nodes=1 << 20, seed=3000):
    """The mesh-packing workload: ``shapes`` rough grains (perturbed
    icospheres of ``frequency``, 20 x frequency^2 triangles) with ``nodes``
    surface sample nodes each, built from ``distinct`` seeded grains repeated
    under their own ids (packing cost does not depend on which grain repeats).
    53 shapes of about a million nodes is the size of the startup whose
    host packing the reference profiles (``docs/RUNTIME_PROFILING.md:62-65``:
    53 shape roots, 2.4 million cluster-tree nodes)."""
    from dataclasses import replace

    from .shapes import ShapeLibrary, perturbed_grain

    rng = np.random.default_rng(seed)
    base = [perturbed_grain(frequency, seed=seed + k, nodes=nodes, axes=rng.uniform(0.6, 1.0, 3))
            for k in range(min(distinct, shapes))]
    return ShapeLibrary([replace(base[k % len(base)], id=f"{base[k % len(base)].id}-copy{k}")
                         for k in range(shapes)])
