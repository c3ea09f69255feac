"""The oracle pinned to the reference's own code and to independent geometry.

* The restated collector against the reference's compiled collector
  (``oracle/_ref/collector_ref.so``, built from the reference tree by
  ``oracle/build_ref.sh``; skipped where that tree is absent): byte-equal
  contact keys, points, normals, per-pair counts and control words.
* Cluster culling against the exhaustive node set
  (``tests/test_cpu_solver.py:794-876``).
* Pair-parallel collection bitwise equal to serial
  (``tests/test_cpu_solver.py:552-632``).
* Mesh distance against an independent FP64 closest-point computation and
  the analytic box distance (``tests/test_mesh_metal.py:23-76``).
"""

import numpy as np
import pytest

from oracle.engine import REF_LIB, OracleEngine, ReferenceCollector
from sand_atlas_dem_gb300.shapes import ShapeLibrary, box_shape, perturbed_grain
from sand_atlas_dem_gb300.spec import Experiment
from tests.specimens import build, lattice_case


def collect(engine):
    c = engine.config(dt=0)
    engine.neighbours(c)
    engine.collect(c)
    ctrl = engine.buffers["control"].copy()
    count = int(ctrl[2])
    side = engine.sides[engine.active]
    return dict(control=ctrl, meta=side["meta"][:count].copy(), point=engine.buffers["pointDepth"][:count].copy(),
                normal=side["normalArea"][:count].copy(), counts=engine.buffers["contactCounts"].copy())


@pytest.mark.skipif(not REF_LIB.exists(), reason="reference collector not built (no reference tree here)")
@pytest.mark.parametrize("frequency,side,seed", [(4, 4, 3), (8, 3, 5), (4, 5, 9)])
def test_restated_collector_equals_reference_collector(frequency, side, seed):
    library, spec, case = lattice_case(side=side, frequency=frequency, seed=seed)
    if side == 3:
        spec.particles = 27
    ours = collect(build(OracleEngine, library, spec, case))
    theirs = collect(build(OracleEngine, library, spec, case, collector=ReferenceCollector()))
    assert int(ours["control"][2]) > 0
    for key in ours:
        assert ours[key].tobytes() == theirs[key].tobytes(), key


@pytest.mark.skipif(not REF_LIB.exists(), reason="reference collector not built (no reference tree here)")
def test_reference_collector_threads_match_restated_threads():
    library, spec, case = lattice_case(side=5, seed=4)
    results = []
    for kwargs in (dict(threads=4), dict(collector=ReferenceCollector(), threads=4)):
        e = build(OracleEngine, library, spec, case, **kwargs)
        e.initialize()
        e.advance(2)
        results.append(e.state())
    for key, value in results[0].items():
        if isinstance(value, np.ndarray):
            assert value.tobytes() == results[1][key].tobytes(), key


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_cluster_cull_equals_exhaustive_node_set(seed):
    library, spec, case = lattice_case(side=4, seed=seed + 20)
    e = build(OracleEngine, library, spec, case)
    culled = collect(e)
    x = build(OracleEngine, library, spec, case)
    c = x.config(dt=0)
    x.neighbours(c)
    x.collect(c, exhaustive=True)
    count = int(x.buffers["control"][2])
    exhaustive = x.sides[x.active]["meta"][:count]

    def keys(meta):
        return meta[np.lexsort(meta[:, :3].T[::-1])]

    assert count > 0
    np.testing.assert_array_equal(keys(culled["meta"]), keys(exhaustive))


def test_parallel_collector_is_bitwise_serial():
    library, spec, case = lattice_case(side=5, seed=7)
    states = []
    for threads in (1, 4):
        e = build(OracleEngine, library, spec, case, threads=threads)
        e.initialize()
        e.advance(3)
        states.append(e.state())
    for key, value in states[0].items():
        if isinstance(value, np.ndarray):
            assert value.tobytes() == states[1][key].tobytes(), key


def probe(engine, shape, points):
    pts = np.zeros((len(points), 4), np.float32)
    pts[:, :3] = points
    out = np.zeros((len(points), 4), np.float32)
    engine.dispatch("meshProbe", len(points), engine.config(), extra=(pts, out), uniforms=(len(points), shape))
    return out


def closest_fp64(vertices, faces, points):
    """Brute-force FP64 unsigned distance to a triangle mesh."""
    tri = vertices[faces]
    best = np.full(len(points), np.inf)
    for a, b, c in tri:
        ab, ac = b - a, c - a
        n = np.cross(ab, ac)
        # Barycentric projection, clamped by edge distances.
        for p_index in range(0, len(points), 4096):
            p = points[p_index:p_index + 4096]
            ap = p - a
            d = np.einsum("ij,j->i", ap, n) / np.dot(n, n)
            proj = p - d[:, None] * n
            v0, v1, v2 = ab, ac, proj - a
            d00, d01, d11 = ab @ ab, ab @ ac, ac @ ac
            d20, d21 = v2 @ ab, v2 @ ac
            den = d00 * d11 - d01 * d01
            v = (d11 * d20 - d01 * d21) / den
            w = (d00 * d21 - d01 * d20) / den
            inside = (v >= 0) & (w >= 0) & (v + w <= 1)
            dist = np.where(inside, np.abs(d) * np.linalg.norm(n), np.inf)
            for s, t in ((a, b), (b, c), (c, a)):
                st = t - s
                u = np.clip(((p - s) @ st) / (st @ st), 0, 1)
                dist = np.minimum(dist, np.linalg.norm(p - (s + u[:, None] * st), axis=1))
            best[p_index:p_index + 4096] = np.minimum(best[p_index:p_index + 4096], dist)
    return best


def test_mesh_distance_matches_fp64_and_analytic_box():
    box = box_shape([1e-3, 2e-3, 3e-3])
    grain = perturbed_grain(4, seed=1000)
    library = ShapeLibrary([box, grain])
    spec = Experiment(particles=2, contact_geometry="mesh", timestep=1e-9)
    e = OracleEngine(library, spec, [[0.005] * 3, [0.015] * 3], [0.03] * 3, [0, 1], [1.0, 1.0])
    rng = np.random.default_rng(79)
    points = np.vstack([rng.uniform(-0.002, 0.002, (513, 3)),
                        [[0.0006, 0, 0], [0.0006, 0.0011, 0], [0.0006, 0.0011, 0.0016], [0, 0, 0], [0.00049, 0, 0]]])
    result = probe(e, 0, points / e.length_unit)
    q = np.abs(points) - [0.0005, 0.001, 0.0015]
    expected = np.linalg.norm(np.maximum(q, 0), axis=1) + np.minimum(q.max(axis=1), 0)
    assert np.max(np.abs(result[:, 3] * e.length_unit - expected)) < 2e-9
    assert np.allclose(np.linalg.norm(result[:, :3], axis=1), 1, atol=2e-5)
    assert np.allclose(result[-4, :3], [2**-0.5, 2**-0.5, 0], atol=2e-5)
    assert np.allclose(result[-3, :3], np.full(3, 3**-0.5), atol=2e-5)
    # Perturbed (non-convex) grain against brute-force FP64 distances.
    pts = rng.uniform(grain.vertices.min(0) * 1.2, grain.vertices.max(0) * 1.2, (257, 3))
    got = probe(e, 1, pts / e.length_unit)[:, 3] * e.length_unit
    dist = closest_fp64(grain.vertices, grain.faces, pts)
    np.testing.assert_allclose(np.abs(got), dist, rtol=2e-4, atol=2e-9)
