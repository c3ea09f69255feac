"""SDF pair contacts against the reference's own FP64 small-case code.

``golden/sdf_pairs.npz`` (written by ``golden/make_sdf_pairs.py``) holds the
reference's ``pair_contact`` (``src/sand_atlas_dem/reference.py:85-172``) for
twelve poses of two rough grains with signed-distance grids: rotated, scaled,
overlapping by 7-24 sample nodes, moving (so the first step's tangential slip
is v_t dt).  The oracle engine, on the same grids and poses with the SDF
contact geometry, must give the same contact count exactly, and the force on
grain i within 2e-5 of its scale and the torques within 5e-5 (measured: 2.0e-6
and 1.2e-5; the engine queries the grids in FP32) -- ten times tighter than
the reference's own tolerance for its solver against ``pair_contact``
(2e-4, ``tests/test_cpu_solver.py:176-209``).
The GPU step equals the oracle bit for bit on the SDF geometry
(``tests/test_gpu_sdf.py``).
"""

from pathlib import Path

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.shapes import Shape, ShapeLibrary
from sand_atlas_dem_gb300.spec import Experiment
from tests.specimens import read, upload

GOLDEN = Path(__file__).resolve().parent / "golden" / "sdf_pairs.npz"
DT = 1e-9


def stored_library(z):
    shapes = []
    for k in range(2):
        f = {name: z[f"shape{k}_{name}"] for name in ("vertices", "faces", "samples", "areas", "sdf", "origin",
                                                       "spacing", "volume", "inertia", "radius")}
        shapes.append(Shape(f"sdf-grain-{k}", f["vertices"], f["faces"].astype(np.int64), f["samples"], f["areas"],
                            float(f["volume"]), f["inertia"], float(f["radius"]), {}, sdf=f["sdf"],
                            origin=f["origin"], spacing=float(f["spacing"])))
    return ShapeLibrary(shapes)


@pytest.fixture(scope="module")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("case", range(12))
def test_sdf_pair_matches_reference_pair_contact(golden, case):
    g = {k[5:]: v[case] for k, v in golden.items() if k.startswith("case_")}
    library = stored_library(golden)
    spec = Experiment(particles=2, contact_geometry="sdf", timestep=DT, friction=float(g["mu"]),
                      max_overlap_fraction=0.5, contacts_per_particle=256, pairs_per_particle=8)
    e = OracleEngine(library, spec, [g["xi"], g["xj"]], [0.01] * 3, [0, 1], [float(g["si"]), float(g["sj"])])
    upload(e, "rotation", np.array([g["qi"], g["qj"]], np.float32))
    v = np.zeros((2, 4), np.float32)
    v[:, :3] = np.array([g["vi"], g["vj"]]) * e.time_unit / e.length_unit
    upload(e, "velocity", v)
    e.initialize()
    assert int(e.check_errors()[2]) == int(g["contacts"])
    force = read(e, "force", 2)[:, :3].astype(float) * e.force_unit
    torque = read(e, "torque", 2)[:, :3].astype(float) * e.energy_unit
    fscale = np.linalg.norm(g["force"])
    tscale = max(np.linalg.norm(g["torque_i"]), np.linalg.norm(g["torque_j"]))
    np.testing.assert_allclose(force[0], g["force"], rtol=0, atol=2e-5 * fscale)
    np.testing.assert_allclose(force[1], -g["force"], rtol=0, atol=2e-5 * fscale)
    np.testing.assert_allclose(torque[0], g["torque_i"], rtol=0, atol=5e-5 * tscale)
    np.testing.assert_allclose(torque[1], g["torque_j"], rtol=0, atol=5e-5 * tscale)
