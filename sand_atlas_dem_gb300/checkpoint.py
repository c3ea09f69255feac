"""Checkpoints and shape libraries in the reference's HDF5 formats, without h5py.

* ``sand-dem-checkpoint/3|4|5`` (``src/sand_atlas_dem/simulation.py:87-136``):
  root attributes (format, step, stage bookkeeping, the experiment as JSON,
  the shape library's SHA-256, backend, initial cell, diagnostic rows, the
  contact count) and one gzip-compressed dataset per ``Engine.state()`` array.
* ``sand-dem-shapes/1`` (``src/sand_atlas_dem/geometry.py:114-163``): root
  attributes format and units, one group per shape (``"0"``, ``"1"``, ...)
  with attributes id, spacing, volume, radius, provenance (JSON) and the
  datasets vertices, faces, samples, areas, sdf, origin, inertia.

Files are read and written by :mod:`sand_atlas_dem_gb300.hdf5`.
"""

import json

import numpy as np

from . import hdf5
from .shapes import Shape, ShapeLibrary
from .spec import Experiment

CHECKPOINT_FORMATS = {"sand-dem-checkpoint/3", "sand-dem-checkpoint/4", "sand-dem-checkpoint/5"}
SHAPES_FORMAT = "sand-dem-shapes/1"
SHAPE_DATASETS = ("vertices", "faces", "samples", "areas", "sdf", "origin", "inertia")


def save_checkpoint(path, engine, *, stage_index=0, stage_steps=0, converged=0, contact_phase=False,
                    filter_stress=(0.0, 0.0, 0.0), rows=(), shape_sha256=""):
    """Write ``engine``'s state as ``Simulation.checkpoint`` does
    (``simulation.py:87-107``); the stage bookkeeping is the caller's."""
    state = engine.state()
    spec = engine.spec
    attrs = dict(
        format=spec.checkpoint_format,
        step=int(engine.step),
        stage_index=int(stage_index),
        stage_steps=int(stage_steps),
        converged=int(converged),
        contact_phase=bool(contact_phase),
        experiment=json.dumps(spec.to_dict()),
        shape_sha256=str(shape_sha256),
        filter_stress=json.dumps([float(v) for v in filter_stress]),
        backend=str(getattr(getattr(engine, "m", None), "name", "gb300")),
        initial_cell=json.dumps(np.asarray(engine.initial_cell, float).tolist()),
        rows=json.dumps(list(rows)),
    )
    members = {}
    for name, value in state.items():
        if name == "contacts":
            attrs[name] = int(value)
        else:
            members[name] = np.asarray(value)
    hdf5.write(path, hdf5.Group(attrs, members), compress=True)


def load_checkpoint(path):
    """The checkpoint's attributes (experiment decoded to an
    :class:`Experiment`) and its state arrays, as ``Simulation.resume``
    reads them (``simulation.py:109-125``)."""
    root = hdf5.read(path)
    if root.attrs.get("format") not in CHECKPOINT_FORMATS:
        raise ValueError("Unsupported checkpoint")
    attrs = dict(root.attrs)
    spec = Experiment(**json.loads(attrs["experiment"]))
    if spec.checkpoint_format != attrs["format"]:
        raise ValueError("Checkpoint boundary version mismatch")
    attrs["experiment"] = spec
    state = {name: np.asarray(root[name]) for name in root}
    state["contacts"] = int(attrs["contacts"])
    return attrs, state


def resume(engine, path):
    """Restore a checkpoint into an engine built for the same experiment,
    library and grains (``simulation.py:126-136``); returns the attributes."""
    attrs, state = load_checkpoint(path)
    engine.initial_cell = np.array(json.loads(attrs["initial_cell"]))
    engine.restore(state, int(attrs["step"]))
    return attrs


def save_shape_library(path, library):
    """``ShapeLibrary.save`` (``geometry.py:114-137``); every shape must carry
    its signed-distance grid, as the format requires."""
    members = {}
    for index, s in enumerate(library.shapes):
        if s.sdf is None:
            raise ValueError("The shape format carries a signed-distance grid on every shape")
        data = {name: np.asarray(getattr(s, name)) for name in SHAPE_DATASETS}
        attrs = dict(id=s.id, spacing=float(s.spacing), volume=float(s.volume), radius=float(s.radius),
                      provenance=json.dumps(s.provenance))
        members[str(index)] = hdf5.Group(attrs, data)
    hdf5.write(path, hdf5.Group(dict(format=SHAPES_FORMAT, units="m"), members), compress=True)


def load_shape_library(path):
    """``ShapeLibrary.load`` (``geometry.py:139-163``)."""
    root = hdf5.read(path)
    if root.attrs.get("format") != SHAPES_FORMAT or root.attrs.get("units") != "m":
        raise ValueError("Unsupported shape format or units")
    shapes = []
    for key in sorted(root, key=int):
        g = root[key]
        s = Shape(str(g.attrs["id"]), g["vertices"], g["faces"], g["samples"], g["areas"], float(g.attrs["volume"]),
                  g["inertia"], float(g.attrs["radius"]), json.loads(g.attrs["provenance"]),
                  sdf=g["sdf"], origin=g["origin"], spacing=float(g.attrs["spacing"]))
        s.validate()
        shapes.append(s)
    return ShapeLibrary(shapes)
