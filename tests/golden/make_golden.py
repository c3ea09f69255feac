"""Regenerates the golden fixtures from the reference implementation itself.

Run in a checkout that has the reference tree (read-only) at
``$SAND_DEM_REFERENCE`` (default /root/reference).  The reference Python
package is imported with stub modules for h5py/trimesh (absent here and not
used by the functions called).  Outputs, committed beside this script:

* ``packing.npz`` — ``mesh.pack_meshes`` arrays for a seeded shape set;
* ``layout.npz``  — the buffers and ``Config`` block the reference ``Engine``
  builds for a seeded 64-grain specimen (through a CPU buffer adapter, no
  kernels run);
* ``packing_trees.npz`` — the tree arrays of ``mesh.pack_meshes`` for shapes
  whose trees have several levels of large nodes (3,000 sample nodes, 2,880
  triangles) and many tied split coordinates (an unperturbed icosphere, its
  nodes rounded to a coarse grid with signed zeros).
"""

import json
import os
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REFERENCE = Path(os.environ.get("SAND_DEM_REFERENCE", "/root/reference"))


def reference_modules():
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    sys.modules.setdefault("trimesh", types.ModuleType("trimesh"))
    os.environ["SAND_DEM_MESH_CACHE"] = "off"
    sys.path.insert(0, str(REFERENCE / "src"))
    import sand_atlas_dem.cpu as cpu
    import sand_atlas_dem.geometry as geometry
    import sand_atlas_dem.gpu as gpu
    import sand_atlas_dem.mesh as mesh
    import sand_atlas_dem.spec as spec

    return cpu, geometry, gpu, mesh, spec


def golden_shapes():
    sys.path.insert(0, str(ROOT))
    from sand_atlas_dem_gb300.shapes import box_shape, exact_cube, perturbed_grain

    return [perturbed_grain(4, seed=1000), perturbed_grain(5, seed=1001, axes=(0.7, 0.9, 1.0)),
            exact_cube(), box_shape([1e-3, 2e-3, 3e-3])]


TREE_ARRAYS = ("meshFrontier", "meshClusterInfo", "meshClusterRanges", "meshClusterMin", "meshClusterMax",
               "meshSampleIndices", "meshRoots", "meshMin", "meshMax", "meshLinks", "meshTriangles")


def tree_shapes():
    """Shapes that stress the median-split trees: deep trees with large nodes,
    and tied coordinates (the stable sort's order) including -0.0 and +0.0."""
    sys.path.insert(0, str(ROOT))
    from sand_atlas_dem_gb300.shapes import Shape, perturbed_grain

    deep = perturbed_grain(12, seed=1002, nodes=3000)
    tied = perturbed_grain(6, seed=1003, sigma=0.0, nodes=1500)
    grid = tied.radius / 8
    samples = np.round(tied.samples / grid) * grid
    samples[::7] *= -1.0  # flips some exact zeros to -0.0
    tied = Shape(tied.id + "-grid", tied.vertices, tied.faces, samples, tied.areas, tied.volume, tied.inertia,
                 tied.radius, dict(tied.provenance))
    return [deep, tied]


def stored_tree_shapes(path=HERE / "packing_trees.npz"):
    """The tree shapes rebuilt from the arrays stored in the fixture (only
    vertices, faces and sample nodes enter the packing)."""
    sys.path.insert(0, str(ROOT))
    from sand_atlas_dem_gb300.shapes import Shape

    shapes = []
    with np.load(path) as z:
        k = 0
        while f"input{k}_vertices" in z.files:
            v, f, s = z[f"input{k}_vertices"], z[f"input{k}_faces"].astype(np.int64), z[f"input{k}_samples"]
            shapes.append(Shape(f"tree-shape-{k}", v, f, s, np.full(len(s), 1e-9), 1e-9, np.eye(3) * 1e-15,
                                float(np.linalg.norm(v, axis=1).max())))
            k += 1
    return shapes


def as_reference_shape(geometry, shape):
    """Reference Shape with a placeholder signed-distance grid (mesh path only)."""
    sdf = np.ones((5, 5, 5), np.float32)
    sdf[2, 2, 2] = -1.0
    return geometry.Shape(shape.id, shape.vertices, shape.faces, shape.samples, shape.areas, sdf,
                          np.full(3, -shape.radius * 1.5), shape.radius * 0.75, shape.volume,
                          shape.inertia, shape.radius, dict(shape.provenance))


class FakeDevice:
    """Buffer-only adapter: the reference Engine constructor allocates, nothing runs."""

    def __init__(self, cpu):
        self.cpu = cpu
        self.device = self

    def buffer(self, array=None, *, count=None, stride=4):
        return self.cpu.Buffer(array, count=count, stride=stride)


def main():
    cpu, geometry, gpu, mesh, spec = reference_modules()
    shapes = golden_shapes()
    library = geometry.ShapeLibrary([as_reference_shape(geometry, s) for s in shapes])
    packed = mesh.pack_meshes(library, 1e-3)
    np.savez_compressed(HERE / "packing.npz", **packed)
    grains = tree_shapes()
    trees = mesh.pack_meshes(geometry.ShapeLibrary([as_reference_shape(geometry, s) for s in grains]), 1e-3)
    # The shapes' own arrays are stored too: regenerating them elsewhere can
    # round differently (BLAS and reductions), and tied coordinates are
    # sensitive to the last bit.
    inputs = {}
    for k, s in enumerate(grains):
        inputs[f"input{k}_vertices"] = s.vertices
        inputs[f"input{k}_faces"] = np.asarray(s.faces, np.int32)
        inputs[f"input{k}_samples"] = s.samples
    np.savez_compressed(HERE / "packing_trees.npz", **{k: trees[k] for k in TREE_ARRAYS}, **inputs)

    from sand_atlas_dem_gb300.workloads import contact_lattice

    grains = geometry.ShapeLibrary([as_reference_shape(geometry, s) for s in shapes[:2]])
    case = contact_lattice(grains, 4, spacing=1.02, seed=11, scale_sigma=0.1)
    experiment = spec.Experiment(particles=64, contact_geometry="mesh", timestep=1e-9, friction=0.4,
                                 normal_viscosity=3e5, contacts_per_particle=64, pairs_per_particle=16)
    e = gpu.Engine(grains, experiment, case["positions"], case["cell"], case["ids"], case["scales"],
                   metal=FakeDevice(cpu))
    out = {f"buffer_{k}": v.array.copy() for k, v in e.buffers.items()}
    config = e.bindings(dt=experiment.timestep)["c"]
    units = {k: getattr(e, k) for k in ("length_unit", "time_unit", "mass_unit", "force_unit", "stress_unit",
                                         "energy_unit", "skin", "cutoff", "pair_capacity", "contact_capacity",
                                         "hash_size", "bin_count", "bin_capacity")}
    units["bins"] = e.bins.tolist()
    np.savez_compressed(HERE / "layout.npz", positions=case["positions"], cell=case["cell"], ids=case["ids"],
                        scales=case["scales"], config=np.array(json.dumps(config)),
                        units=np.array(json.dumps(units, default=float)), **out)
    print("wrote", HERE / "packing.npz", HERE / "layout.npz", HERE / "packing_trees.npz")


if __name__ == "__main__":
    main()
