"""Golden vectors of the per-contact law from the reference's own FP64 code.

Run in a checkout that has the reference tree (read-only) at
``$SAND_DEM_REFERENCE`` (default /root/reference).  Calls the reference's
independent FP64 small-case functions (``src/sand_atlas_dem/reference.py``):

* ``nodal_force`` (``reference.py:69-82``): the half-weighted directed traction
  law -- normal force 0.5 kn A delta, trial slip over the step, tangential
  traction -0.5 kt A slip with its Coulomb cap -- returning the force and the
  new elastic slip;
* ``transport_slip`` (``reference.py:48-66``): the elastic slip carried from
  the previous contact normal to the new one (minimal rotation) and turned by
  the mean spin about it.

Writes ``contact_law.npz`` beside this script: seeded inputs (normalized
units; sliding and sticking contacts, some with no overlap) and the
reference's outputs in float64.
"""

import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REFERENCE = Path(os.environ.get("SAND_DEM_REFERENCE", "/root/reference"))


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def law_cases(rng, n=512):
    normal = unit(rng, n)
    depth = 10 ** rng.uniform(-5, -2, n)
    depth[:16] = -depth[:16]  # no overlap: no force
    area = 10 ** rng.uniform(-3, 0, n)
    slip = unit(rng, n) * 10 ** rng.uniform(-6, -2, n)[:, None]
    velocity = unit(rng, n) * 10 ** rng.uniform(-4, 0, n)[:, None]
    kn = 1.0
    kt = 0.5
    mu = np.where(rng.random(n) < 0.15, 0.0, rng.choice([0.05, 0.3, 0.5, 1.0], n))
    dt = 10 ** rng.uniform(-3, -1, n)
    return dict(normal=normal, depth=depth, area=area, slip=slip, velocity=velocity, kn=np.full(n, kn),
                kt=np.full(n, kt), mu=mu, dt=dt)


def transport_cases(rng, n=384):
    old = unit(rng, n)
    new = unit(rng, n)
    # Keep away from the flipped-normal cut (the reference and the production
    # kernels place it at slightly different cosines).
    flip = np.einsum("ij,ij->i", old, new) < -0.9
    new[flip] = -new[flip]
    slip = rng.normal(size=(n, 3)) * 1e-3
    spin = rng.uniform(-0.2, 0.2, n)
    spin[:32] = 0.0
    return dict(slip=slip, old=old, new=new, spin=spin)


def main():
    # The package imports h5py/trimesh at module level; neither is used here.
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    sys.modules.setdefault("trimesh", types.ModuleType("trimesh"))
    os.environ["SAND_DEM_MESH_CACHE"] = "off"
    sys.path.insert(0, str(REFERENCE / "src"))
    from sand_atlas_dem.reference import nodal_force, transport_slip

    rng = np.random.default_rng(2026)
    law = law_cases(rng)
    force = np.zeros((len(law["depth"]), 3))
    new_slip = np.zeros_like(force)
    for k in range(len(force)):
        f, s = nodal_force(law["depth"][k], law["normal"][k], law["area"][k], law["slip"][k], law["velocity"][k],
                           law["kn"][k], law["kt"][k], law["mu"][k], law["dt"][k])
        force[k], new_slip[k] = f, s
    moved = transport_cases(rng)
    carried = np.array([transport_slip(moved["slip"][k], moved["old"][k], moved["new"][k], moved["spin"][k])
                        for k in range(len(moved["spin"]))])
    np.savez_compressed(HERE / "contact_law.npz", **{f"law_{k}": v for k, v in law.items()},
                        **{f"transport_{k}": v for k, v in moved.items()}, out_force=force, out_slip=new_slip,
                        out_transport=carried)
    print("wrote", HERE / "contact_law.npz", "cases", len(force), "+", len(carried))


if __name__ == "__main__":
    main()
