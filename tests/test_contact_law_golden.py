"""The oracle's per-contact law against the reference's own FP64 code.

``golden/contact_law.npz`` (written by ``golden/make_contact_law.py``) holds
the outputs of the reference's independent FP64 functions ``nodal_force`` and
``transport_slip`` (``src/sand_atlas_dem/reference.py:48-82``) on seeded
contacts: sticking and sliding, with and without overlap, slips carried
between normals with and without spin.  The oracle evaluates the same cases
through the functions its ``resolveContacts`` calls (``grainLaw`` with no
normal viscosity, ``transported``; probes ``grainLawProbe``,
``transportProbe``): its FP64 build must agree to 1e-14 of each result's
scale (measured: 7e-16), its FP32 build (the one the GPU step equals bit for
bit) to 2e-6 (measured: 6e-7).
"""

from pathlib import Path

import numpy as np
import pytest

from oracle.engine import OracleEngine
from sand_atlas_dem_gb300.shapes import ShapeLibrary, box_shape
from sand_atlas_dem_gb300.spec import Experiment

GOLDEN = Path(__file__).resolve().parent / "golden" / "contact_law.npz"


def engine(precision):
    spec = Experiment(particles=2, contact_geometry="mesh", timestep=1e-9)
    library = ShapeLibrary([box_shape([1e-3, 1e-3, 1e-3])])
    return OracleEngine(library, spec, [[0.005] * 3, [0.015] * 3], [0.03] * 3, [0, 0], [1.0, 1.0],
                        precision=precision)


def rows(real, xyz, w=None):
    out = np.zeros((len(xyz), 4), real)
    out[:, :3] = xyz
    if w is not None:
        out[:, 3] = w
    return out


def law(e, real, g, mu, dt):
    n = len(g["law_mu"])
    normal_depth = rows(real, g["law_normal"], g["law_depth"])
    slip_area = rows(real, g["law_slip"], g["law_area"])
    velocity = rows(real, g["law_velocity"])
    force, slip = np.zeros((n, 4), real), np.zeros((n, 4), real)
    e.dispatch("grainLawProbe", n, e.config(), extra=(normal_depth, slip_area, velocity, force, slip),
               uniforms=(n, g["law_kn"][0], g["law_kt"][0], mu, 0.0, dt))
    return force[:, :3], slip[:, :3]


@pytest.mark.parametrize("precision,tolerance", [("fp64", 1e-14), ("fp32", 2e-6)])
def test_grain_law_matches_reference_nodal_force(precision, tolerance):
    with np.load(GOLDEN) as z:
        g = {k: z[k] for k in z.files}
    real = np.float64 if precision == "fp64" else np.float32
    e = engine(precision)
    # The probe takes one (mu, dt) a call: group the cases by them.
    for k in range(len(g["law_mu"])):
        one = {name: (v[k:k + 1] if name.startswith("law_") else v) for name, v in g.items()}
        force, slip = law(e, real, one, float(g["law_mu"][k]), float(g["law_dt"][k]))
        ref_force, ref_slip = g["out_force"][k], g["out_slip"][k]
        fscale = 0.5 * g["law_kn"][k] * g["law_area"][k] * abs(g["law_depth"][k]) + np.linalg.norm(ref_force)
        sscale = np.linalg.norm(g["law_slip"][k]) + np.linalg.norm(g["law_velocity"][k]) * g["law_dt"][k]
        assert np.all(np.abs(force[0] - ref_force) <= tolerance * fscale + 1e-300), (k, force, ref_force)
        assert np.all(np.abs(slip[0] - ref_slip) <= tolerance * sscale + 1e-300), (k, slip, ref_slip)


@pytest.mark.parametrize("precision,tolerance", [("fp64", 1e-14), ("fp32", 2e-6)])
def test_slip_transport_matches_reference(precision, tolerance):
    with np.load(GOLDEN) as z:
        g = {k: z[k] for k in z.files}
    real = np.float64 if precision == "fp64" else np.float32
    e = engine(precision)
    n = len(g["transport_spin"])
    slip_spin = rows(real, g["transport_slip"], g["transport_spin"])
    old, new = rows(real, g["transport_old"]), rows(real, g["transport_new"])
    result = np.zeros((n, 4), real)
    e.dispatch("transportProbe", n, e.config(), extra=(slip_spin, old, new, result), uniforms=(n,))
    scale = np.linalg.norm(g["transport_slip"], axis=1, keepdims=True)
    assert np.all(np.abs(result[:, :3] - g["out_transport"]) <= tolerance * scale)
