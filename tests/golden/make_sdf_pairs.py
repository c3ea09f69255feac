"""Golden SDF pair contacts from the reference's own FP64 small-case code.

Run in a checkout that has the reference tree (read-only) at
``$SAND_DEM_REFERENCE`` (default /root/reference).  For two rough grains with
signed-distance grids (perturbed icospheres, ``shapes.with_sdf``, the
reference's grid layout) at seeded poses -- rotated, scaled, overlapping,
moving -- calls the reference's ``pair_contact``
(``src/sand_atlas_dem/reference.py:85-172``: both directions, every sample node
of one grain queried on the other's grid in FP64, ``nodal_force`` per node)
and stores the pair's force on grain i, the torques on both grains and the
contact count.  The shapes' own arrays are stored as well, so the cases do not
depend on regenerating them.  Writes ``sdf_pairs.npz`` beside this script.
"""

import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REFERENCE = Path(os.environ.get("SAND_DEM_REFERENCE", "/root/reference"))
SHAPE_FIELDS = ("vertices", "faces", "samples", "areas", "sdf", "origin", "spacing", "volume", "inertia", "radius")
KN, KT, DT = 1e12, 5e11, 1e-9


def grains():
    sys.path.insert(0, str(ROOT))
    from sand_atlas_dem_gb300.shapes import perturbed_grain, with_sdf

    return [with_sdf(perturbed_grain(4, seed=1400 + k), resolution=16) for k in range(2)]


def unit_quaternion(rng):
    q = rng.normal(size=4)
    return q / np.linalg.norm(q)


def main():
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    sys.modules.setdefault("trimesh", types.ModuleType("trimesh"))
    os.environ["SAND_DEM_MESH_CACHE"] = "off"
    sys.path.insert(0, str(REFERENCE / "src"))
    from sand_atlas_dem.geometry import Shape
    from sand_atlas_dem.reference import pair_contact

    shapes = grains()
    ref = [Shape(s.id, s.vertices, s.faces, s.samples, s.areas, s.sdf, s.origin, s.spacing, s.volume, s.inertia,
                 s.radius, dict(s.provenance)) for s in shapes]
    rng = np.random.default_rng(77)
    cases = {k: [] for k in ("xi", "xj", "qi", "qj", "si", "sj", "vi", "vj", "mu", "force", "torque_i", "torque_j",
                             "contacts")}
    while len(cases["mu"]) < 12:
        si, sj = rng.uniform(0.9, 1.1, 2)
        qi, qj = unit_quaternion(rng), unit_quaternion(rng)
        direction = rng.normal(size=3)
        direction /= np.linalg.norm(direction)
        distance = (shapes[0].radius * si + shapes[1].radius * sj) * rng.uniform(0.7, 0.88)
        xi = np.full(3, 0.005)
        xj = xi + distance * direction
        vi, vj = rng.normal(size=3) * 0.05, rng.normal(size=3) * 0.05
        mu = float(rng.choice([0.1, 0.5]))
        r = pair_contact(ref[0], ref[1], xi, xj, qi=qi, qj=qj, si=si, sj=sj, kn=KN, kt=KT, mu=mu, vi=vi, vj=vj,
                         dt=DT)
        if r["contacts"] < 4:
            continue
        for name, value in (("xi", xi), ("xj", xj), ("qi", qi), ("qj", qj), ("si", si), ("sj", sj), ("vi", vi),
                            ("vj", vj), ("mu", mu), ("force", r["force"]), ("torque_i", r["torque_i"]),
                            ("torque_j", r["torque_j"]), ("contacts", r["contacts"])):
            cases[name].append(value)
    arrays = {f"case_{k}": np.asarray(v) for k, v in cases.items()}
    for index, s in enumerate(shapes):
        for field in SHAPE_FIELDS:
            arrays[f"shape{index}_{field}"] = np.asarray(getattr(s, field))
    np.savez_compressed(HERE / "sdf_pairs.npz", **arrays)
    print("wrote", HERE / "sdf_pairs.npz", len(cases["mu"]), "cases, contacts", cases["contacts"])


if __name__ == "__main__":
    main()
