"""CUDA step against the CPU oracle at the benchmarked configurations.

The small-lattice parity tests run 320-triangle shapes; these run the shapes,
packings and paths the benchmark measures, on the default (accelerated)
engine: certified distance-bound grid, stored node-filter results and walk
certificates.

* the committed dense 10,000-grain packing of the 1,280-triangle library
  (the ``dense-10k`` workload, its material and timestep);
* a 1,728-grain lattice of the uneven library at solid fraction 0.58 with a
  quarter of the grains on the 5,120-triangle shape and a quarter on the
  4,500-triangle shapes;
* a batch of three uneven-library specimens against one oracle run per
  specimen (the reference has one specimen per engine, ``gpu.py:95-97``).

Gates (the contract of the reference CPU backend comparison): pair lists,
contact keys and their order bit-exact, contact geometry and forces bit-exact
at the zero-timestep initialization; after timesteps forces, torques, poses
and slips within 1e-5 relative with identical contact keys; and from an
identical state (the GPU's own, restored into both) the history slot map is
bit-exact: the slips the contact law carries forward and the forces are equal
byte for byte.  The oracle runs multi-threaded on the host cores.
"""

import os
from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.engine import Engine
from sand_atlas_dem_gb300.shapes import synthetic_library
from sand_atlas_dem_gb300.workloads import lattice_at, load_packing, material_spec

pytestmark = pytest.mark.gpu
REL = 1e-5
THREADS = os.cpu_count() or 1
PACKING = Path(__file__).resolve().parent.parent / "sand_atlas_dem_gb300" / "data" / "packing-f8-10000.npz"
_LIBRARIES = {}


def library(kind):
    if kind not in _LIBRARIES:
        _LIBRARIES[kind] = synthetic_library(kind, 64)
    return _LIBRARIES[kind]


def assert_close(a, b, what):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    err = np.abs(a - b).max() if a.size else 0.0
    assert err <= REL * scale, f"{what}: max error {err:.3e} vs scale {scale:.3e}"


def make(cls, lib, spec, case, **kwargs):
    e = cls(lib, spec, case["positions"], case["cell"], case["ids"], case["scales"], **kwargs)
    rotations = np.ascontiguousarray(case["rotations"], np.float32)
    if isinstance(e.buffers["rotation"], np.ndarray):
        e.buffers["rotation"][...] = rotations
    else:
        e.buffers["rotation"].copy_from_numpy(rotations)
    return e


def committed(e, name, count, dtype=np.float32):
    side = e.sides[1 - e.active]
    if isinstance(side[name], np.ndarray):
        return side[name][:count]
    return e.m.read_prefix(side[name], 4 * count, dtype, shape=(count, 4))


def current(e, name, rows, dtype=np.float32, width=4):
    buffer = e.buffers[name]
    if isinstance(buffer, np.ndarray):
        return buffer.reshape(-1, width)[:rows]
    return e.read(name, dtype, (rows, width))


def assert_initialized_identically(o, g):
    oc, gc = o.check_errors(), g.check_errors()
    pairs, count = int(oc[1]), int(oc[2])
    assert (int(gc[1]), int(gc[2])) == (pairs, count) and count > 0
    np.testing.assert_array_equal(current(g, "pairs", pairs, np.uint32, 2), o.buffers["pairs"][:pairs])
    assert committed(g, "meta", count, np.uint32).tobytes() == committed(o, "meta", count, np.uint32).tobytes()
    assert committed(g, "normalArea", count).tobytes() == committed(o, "normalArea", count).tobytes()
    for name in ("pointDepth", "contactForce"):
        assert current(g, name, count).tobytes() == o.buffers[name][:count].tobytes(), name
    n = o.n
    for name, rows in (("force", n), ("torque", n), ("particleStress", 3 * n), ("particleDiagnostic", n)):
        assert current(g, name, rows).tobytes() == o.buffers[name][:rows].tobytes(), name
    return pairs, count


def assert_steps_agree(o, g, chunks, rate):
    for chunk in chunks:
        o.advance(chunk, rate=rate)
        g.advance(chunk, rate=rate)
        so, sg = o.state(), g.state()
        assert so["contacts"] == sg["contacts"]
        np.testing.assert_array_equal(sg["meta"], so["meta"])
        for name in ("position", "velocity", "rotation", "momentum", "force", "torque", "slip", "normalArea"):
            assert_close(sg[name], so[name], name)
    return sg


def assert_history_map_identical(lib, spec, case, state, step, o_kwargs):
    """Both engines restart from the same state: the contacts they collect,
    the slips their history lookups carry forward and the forces agree bit
    for bit (the new->old slot map is the same)."""
    o = make(OracleEngine, lib, spec, case, **o_kwargs)
    g = make(Engine, lib, spec, case)
    o.restore(state, step)
    g.restore(state, step)
    so, sg = o.state(), g.state()
    assert so["contacts"] == sg["contacts"] > 0
    np.testing.assert_array_equal(sg["meta"], so["meta"])
    for name in ("slip", "normalArea", "force", "torque"):
        assert sg[name].tobytes() == so[name].tobytes(), name
    # Some carried slips are nonzero: the map is exercised, not vacuous.
    assert np.abs(so["slip"][:, :3]).max() > 0


def dense_case():
    pack = load_packing(PACKING)
    lib = library("f8")
    spec = material_spec(lib, pack["ids"], pack["scales"], max_overlap_fraction=0.1)
    return lib, spec, pack


def test_dense_10k_packing_matches_oracle(gpu_library):
    lib, spec, case = dense_case()
    o = make(OracleEngine, lib, spec, case, threads=THREADS)
    g = make(Engine, lib, spec, case)
    assert g.filter_margin > 0 and g.distance_grid  # the benchmarked, accelerated path
    o.initialize()
    g.initialize()
    pairs, count = assert_initialized_identically(o, g)
    assert pairs > 50_000 and count > 100_000
    state = assert_steps_agree(o, g, (1, 2), (-0.5, -0.5, -0.5))
    assert_history_map_identical(lib, spec, case, state, g.step, dict(threads=THREADS))


def uneven_case(side=12, seed=5):
    lib = library("uneven")
    case = lattice_at(lib, side, 0.58, seed=seed)
    tris = np.array([len(s.faces) for s in lib.shapes])
    rng = np.random.default_rng(seed)
    n = side**3
    pick = rng.permutation(n)
    ids = case["ids"].copy()
    ids[pick[: n // 4]] = int(np.argmax(tris))
    ids[pick[n // 4: n // 2]] = rng.choice(np.flatnonzero(tris == 4500), n // 2 - n // 4)
    case["ids"] = ids
    spec = material_spec(lib, ids, case["scales"], max_overlap_fraction=0.5, pairs_per_particle=16,
                         contacts_per_particle=384)
    return lib, spec, case, tris


def test_uneven_library_with_5120_triangle_shapes_matches_oracle(gpu_library):
    lib, spec, case, tris = uneven_case()
    o = make(OracleEngine, lib, spec, case, threads=THREADS)
    g = make(Engine, lib, spec, case)
    o.initialize()
    g.initialize()
    _, count = assert_initialized_identically(o, g)
    meta = committed(o, "meta", count, np.uint32)
    targets = tris[case["ids"][meta[:, 1]]]
    assert (targets == 5120).sum() > 1000 and (targets == 4500).sum() > 1000
    state = assert_steps_agree(o, g, (1, 2), (-0.5, -0.5, -0.5))
    assert_history_map_identical(lib, spec, case, state, g.step, dict(threads=THREADS))


def batch_specimens():
    """Three uneven-library lattices.  Each holds one copy of the batch's
    largest grain (the widest shape at the largest scale), so every specimen
    alone has the batch's Verlet skin, cutoff and bin grid, and its pair list
    alone equals its part of the batch's."""
    lib = library("uneven")
    cases = [lattice_at(lib, side, phi, seed=seed) for side, phi, seed in ((6, 0.58, 21), (7, 0.56, 22), (8, 0.6, 23))]
    radius = np.array([s.radius for s in lib.shapes])
    widest = int(np.argmax(radius))
    top = max(float(c["scales"].max()) for c in cases)
    for c in cases:
        c["ids"] = c["ids"].copy()
        c["scales"] = c["scales"].copy()
        c["ids"][0], c["scales"][0] = widest, top
    return lib, cases


def test_batch_matches_oracle_per_specimen(gpu_library):
    lib, cases = batch_specimens()
    counts = [len(c["positions"]) for c in cases]
    starts = np.cumsum([0] + counts)
    ids = np.concatenate([c["ids"] for c in cases])
    scales = np.concatenate([c["scales"] for c in cases])
    spec = material_spec(lib, ids, scales, max_overlap_fraction=0.5, pairs_per_particle=16, contacts_per_particle=384)
    rates = np.array([[-0.5, -0.5, -0.5], [-0.1, -0.2, -0.3], [0.0, 0.0, -1.0]])
    batch = Engine.batch(lib, spec, [(c["positions"], c["cell"], c["ids"], c["scales"]) for c in cases])
    batch.buffers["rotation"].copy_from_numpy(np.concatenate([c["rotations"] for c in cases]).astype(np.float32))
    oracles = []
    for c, n in zip(cases, counts):
        o = make(OracleEngine, lib, replace(spec, particles=n), c, threads=THREADS)
        assert o.layout.cutoff == batch.layout.cutoff and o.layout.skin == batch.layout.skin
        oracles.append(o)
    batch.initialize()
    for o in oracles:
        o.initialize()
    ctrl = batch.check_errors()
    pairs = current(batch, "pairs", int(ctrl[1]), np.uint32, 2)
    meta = committed(batch, "meta", int(ctrl[2]), np.uint32)
    force = current(batch, "force", batch.n)
    for k, o in enumerate(oracles):
        lo, hi = starts[k], starts[k + 1]
        oc = o.check_errors()
        mine = pairs[(pairs[:, 0] >= lo) & (pairs[:, 0] < hi)] - np.uint32(lo)
        np.testing.assert_array_equal(mine, o.buffers["pairs"][: int(oc[1])])
        rows = meta[(meta[:, 0] >= lo) & (meta[:, 0] < hi)].copy()
        rows[:, :2] -= np.uint32(lo)
        # Same keys in the same order (pair, direction, leaf preorder, node).
        np.testing.assert_array_equal(rows, committed(o, "meta", int(oc[2]), np.uint32))
        assert force[lo:hi].tobytes() == o.buffers["force"][: hi - lo].tobytes()
    for chunk in (1, 2):
        batch.advance(chunk, rate=rates)
        for k, o in enumerate(oracles):
            o.advance(chunk, rate=tuple(rates[k]))
    sb = batch.state()
    for k, o in enumerate(oracles):
        lo, hi = starts[k], starts[k + 1]
        so = o.state()
        rows = (sb["meta"][:, 0] >= lo) & (sb["meta"][:, 0] < hi)
        mine = sb["meta"][rows].copy()
        mine[:, :2] -= np.uint32(lo)
        np.testing.assert_array_equal(mine, so["meta"])
        np.testing.assert_array_equal(sb["cell"][3 * k:3 * k + 3], so["cell"])
        for name in ("position", "velocity", "rotation", "force", "torque"):
            assert_close(sb[name][lo:hi], so[name], f"specimen {k} {name}")
        assert_close(sb["slip"][rows], so["slip"], f"specimen {k} slip")
