"""Backend selection: ``"gb300"`` as a third backend value beside the reference's.

The reference chooses its compute backend in ``Simulation.__init__``
(``src/sand_atlas_dem/simulation.py:60-68``): ``backend=None`` or
``"metal"`` runs its Metal adapter, ``"cpu"`` its generated-C++ CPU adapter,
and any other value raises ``ValueError``; there is no automatic fallback
(``backend.py:1``, ``cpu.py:1-5``).  :func:`with_gb300` returns a subclass
of a ``Simulation`` class (the reference's, passed in: this package neither
imports nor modifies the reference) that also accepts ``backend="gb300"``
and then steps the whole laboratory -- stages, servo, diagnostics rows,
checkpoints -- on :class:`sand_atlas_dem_gb300.engine.Engine`.  The
reference's own ``__init__`` runs unchanged (initial assembly, orientations,
``initialize``); only the engine class it constructs is this one.
``Simulation.resume`` needs nothing more: it passes the checkpoint's
``backend`` attribute (the engine's ``m.name``, ``"gb300"``) back to the
constructor (``simulation.py:110-136``).
"""

import sys
import threading

BACKENDS = (None, "metal", "cpu", "gb300")
_SWAP = threading.Lock()


def select(backend):
    """The reference's rule with ``"gb300"`` added: one of :data:`BACKENDS`."""
    if backend not in BACKENDS:
        raise ValueError("Backend must be explicitly metal, cpu or gb300")
    return backend


def _engine_class():
    from .engine import Engine

    return Engine


def with_gb300(simulation_cls, engine_cls=None):
    """A subclass of ``simulation_cls`` whose constructor also accepts
    ``backend="gb300"``.

    ``engine_cls`` (default :class:`~sand_atlas_dem_gb300.engine.Engine`) is
    constructed with the reference ``Engine``'s arguments ``(library,
    experiment, positions, cell, shape_ids, scales)``.  The other backend
    values go to the reference's constructor untouched.
    """
    module = sys.modules[simulation_cls.__module__]
    if not hasattr(module, "Engine"):
        raise TypeError("the Simulation's module constructs no Engine")

    class GB300Simulation(simulation_cls):
        def __init__(self, experiment, *, library=None, metal=None, backend=None):
            select(backend)
            if backend != "gb300":
                super().__init__(experiment, library=library, metal=metal, backend=backend)
                return
            if metal is not None:
                raise ValueError("Cannot combine GB300 selection with a Metal device")
            engine = engine_cls or _engine_class()

            def construct(library, experiment, positions, cell, ids, scales, metal=None):
                return engine(library, experiment, positions, cell, ids, scales)

            # The reference constructor looks `Engine` up in its module at
            # call time: it builds this engine for the duration of the call.
            with _SWAP:
                reference_engine = module.Engine
                module.Engine = construct
                try:
                    super().__init__(experiment, library=library, metal=None, backend=None)
                finally:
                    module.Engine = reference_engine

    GB300Simulation.__name__ = GB300Simulation.__qualname__ = simulation_cls.__name__
    GB300Simulation.__module__ = __name__
    return GB300Simulation
