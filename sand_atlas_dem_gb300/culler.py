"""Learned conservative culler for the exact node query (no reference counterpart).

One small signed-distance network per shape,
``h0 = sin(W0 p + b0)``, ``h1 = relu(W1 h0 + b1)``, ``y = w2 . h1 + b2``
(3 -> 64 Fourier features -> 64 -> 1), trained on the GPU by this
package's own forward/backward kernels (``csrc/culler.cu``) on points
uniform in a shell of +-``shell`` around each surface and, a quarter as many,
uniform in the interior, labelled by the exact BVH distance the contact query
itself computes.  At run time the hidden
layer runs on tensor cores (BF16 weights, FP32 accumulation, ``csrc/
culler.cuh``) inside the node-query warps.

Conservative by construction of its margins: a node is skipped only when
its prediction exceeds its cell's margin -- per cell of an 8^3 grid over the
shape's root box, the largest prediction at any of (3 x points) sampled
inside points (the inside half of the shell, the whole interior and the
surface itself, fresh seeds) in the cell and its neighbours, plus ``slack``,
and never above the whole shape's margin.  Every other node takes the exact query, which alone
decides contacts and forces.  Missed contacts are counted against the exact
path by the tests.
"""

import ctypes as ct

import numpy as np

from . import native

H = 64
CELLS = 8  # margin cells per axis of each shape's root box (csrc CULLER_CELLS)


def _decode(keys):
    """Ordered integers (sdg_culler_inside_max) back to floats."""
    k = np.asarray(keys).view(np.uint32)
    bits = np.where(k & 0x80000000, k ^ 0x80000000, ~k).astype(np.uint32)
    return bits.view(np.float32)


def _torch():
    import torch

    return torch


def _ptr(t):
    return ct.c_void_p(t.data_ptr())


def _engine_stream(method):
    """Run a method with the engine stream current, so that torch's
    allocations, fills and reads are ordered with the kernels launched on it."""
    import functools

    @functools.wraps(method)
    def wrapped(self, *args, **kwargs):
        with _torch().cuda.stream(self.stream):
            return method(self, *args, **kwargs)

    return wrapped


class LearnedCuller:
    """Per-shape networks for one engine's shape library."""

    def __init__(self, engine, *, shell=0.3, points=1 << 20, steps=2000, batch=8192, lr=1e-3, seed=7,
                 slack=0.05, over=20.0, min_cell_samples=256):
        self.engine = engine
        self.lib = native.load()
        self.shapes = len(engine.library.shapes)
        self.params_per_shape = self.lib.sdg_culler_param_count()
        radii = np.array([s.radius for s in engine.library.shapes]) / engine.length_unit
        self.shell = float(shell * np.median(radii))  # normalized units
        self.points, self.steps, self.batch, self.lr, self.seed, self.slack = points, steps, batch, lr, seed, slack
        self.over = float(over)  # weight of an over-prediction inside a shape in the training loss
        self.min_cell_samples = int(min_cell_samples)
        self.cell_margins = None
        torch = _torch()
        self.device = engine.device
        self.stream = engine.stream
        with torch.cuda.stream(self.stream):
            self.params = torch.from_numpy(self.initial_params()).to(self.device)
            self.w1 = torch.zeros(self.shapes * H * H, dtype=torch.int16, device=self.device)
        self.margins = None
        self.losses = []

    def initial_params(self):
        """Seeded initialization: Fourier frequencies N(0, (3/shell)^2 ... ) scaled to the shell."""
        rng = np.random.default_rng(self.seed)
        p = np.zeros((self.shapes, self.params_per_shape), np.float32)
        w0 = 3 * H
        for s in range(self.shapes):
            p[s, :w0] = rng.normal(0.0, 1.0 / self.shell, w0)
            p[s, w0:w0 + H] = rng.uniform(-np.pi, np.pi, H)
            p[s, 256:256 + H * H] = rng.normal(0.0, np.sqrt(2.0 / H), H * H)
            p[s, 256 + H * H + H:256 + H * H + 2 * H] = rng.normal(0.0, np.sqrt(1.0 / H), H)
        return p

    # ------------------------------------------------------------ data
    @_engine_stream
    def sample(self, count, seed, *, inside_only=False):
        """``count`` accepted points per shape (x, y, z, phi), exact labels."""
        torch = _torch()
        e = self.engine
        candidates = 4 * count
        out = torch.zeros((self.shapes * candidates, 4), dtype=torch.float32, device=self.device)
        accept = torch.zeros(self.shapes * candidates, dtype=torch.int32, device=self.device)
        ptrs, sizes = e._arrays(e.active)
        values, nv = e._values(e.config())
        s = ct.c_void_p(self.stream.cuda_stream)
        native.check(self.lib.sdg_culler_sample(ptrs, sizes, values, nv, self.shapes, candidates, seed,
                                                self.shell, int(inside_only), _ptr(out), _ptr(accept), s))
        offsets = torch.zeros(self.shapes * candidates, dtype=torch.int32, device=self.device)
        partials = torch.zeros(self.lib.sdg_scan_partials(), dtype=torch.int32, device=self.device)
        native.check(self.lib.sdg_exclusive_scan(_ptr(accept), _ptr(offsets), self.shapes * candidates, None,
                                                 _ptr(partials), s))
        points = torch.zeros((self.shapes * count, 4), dtype=torch.float32, device=self.device)
        native.check(self.lib.sdg_culler_compact(_ptr(out), _ptr(accept), _ptr(offsets), self.shapes, candidates,
                                                 count, _ptr(points), s))
        self.stream.synchronize()
        accepted = accept.view(self.shapes, candidates).sum(dim=1).cpu().numpy()
        if accepted.min() < count:
            raise RuntimeError(f"shell sampling accepted only {accepted.min()} of {count} points for a shape")
        return points

    # ---------------------------------------------------------- training
    @_engine_stream
    def train(self, log=None):
        torch = _torch()
        # The shell (where the decisions are made) and, a quarter as many,
        # the deep interior, so that predictions there are negative too.
        shell = self.sample(self.points, self.seed).view(self.shapes, self.points, 4)
        inside = self.sample(self.points // 4, self.seed + 17, inside_only=True).view(self.shapes, -1, 4)
        self.training_points = torch.cat([shell, inside], dim=1).reshape(-1, 4).contiguous()
        per_shape = self.training_points.shape[0] // self.shapes
        n = self.shapes * self.params_per_shape
        grads = torch.zeros(n, dtype=torch.float32, device=self.device)
        m = torch.zeros_like(grads)
        v = torch.zeros_like(grads)
        rows = self.shapes * self.batch
        scratch = torch.zeros(4 * rows * H + 3 * rows, dtype=torch.float32, device=self.device)
        loss = torch.zeros(rows, dtype=torch.float32, device=self.device)
        s = ct.c_void_p(self.stream.cuda_stream)
        for step in range(self.steps):
            lr = self.lr * (0.1 ** (step / max(1, self.steps)))
            native.check(self.lib.sdg_culler_train_step(
                _ptr(self.params), _ptr(self.training_points), self.shapes, per_shape, self.batch, step,
                self.seed, self.shell, self.over, lr, _ptr(grads), _ptr(m), _ptr(v), _ptr(scratch),
                ct.cast(ct.c_void_p(loss.data_ptr()), ct.POINTER(ct.c_float)), s))
            if step % 100 == 0 or step == self.steps - 1:
                self.stream.synchronize()
                mse = float(loss.view(self.shapes, self.batch).mean())
                self.losses.append((step, mse))
                if log:
                    log(dict(step=step, mse=mse))
        self.stream.synchronize()
        return self.losses

    @_engine_stream
    def gradients(self, step=0):
        """Parameter gradients of the mean squared error on batch ``step``."""
        torch = _torch()
        grads = torch.zeros(self.shapes * self.params_per_shape, dtype=torch.float32, device=self.device)
        rows = self.shapes * self.batch
        scratch = torch.zeros(4 * rows * H + 3 * rows, dtype=torch.float32, device=self.device)
        per_shape = self.training_points.shape[0] // self.shapes
        native.check(self.lib.sdg_culler_gradients(
            _ptr(self.params), _ptr(self.training_points), self.shapes, per_shape, self.batch, step, self.seed,
            self.shell, self.over, _ptr(grads), _ptr(scratch), ct.c_void_p(self.stream.cuda_stream)))
        self.stream.synchronize()
        index = scratch[4 * rows * H + 2 * rows:].view(torch.int32)[:rows].cpu().numpy().view(np.uint32)
        return grads.view(self.shapes, -1).cpu().numpy(), index.reshape(self.shapes, self.batch)

    # ------------------------------------------------------- calibration
    @_engine_stream
    def predict(self, points):
        """Run-time (tensor-core) predictions for stored points (shapes x count)."""
        torch = _torch()
        count = points.shape[0] // self.shapes
        out = torch.zeros(self.shapes * count, dtype=torch.float32, device=self.device)
        native.check(self.lib.sdg_culler_tile_eval(_ptr(self.params), _ptr(self.w1), _ptr(points), self.shapes,
                                                   count, _ptr(out), ct.c_void_p(self.stream.cuda_stream)))
        self.stream.synchronize()
        if bool(torch.isnan(out).any()):
            raise RuntimeError("culler: a tensor-core wait gave up")
        return out

    @_engine_stream
    def evaluate(self, points):
        """The same function on CUDA cores: FP32 rows, BF16 features and hidden
        weights (the tensor-core tile's reference for tests)."""
        torch = _torch()
        count = points.shape[0] // self.shapes
        out = torch.zeros(self.shapes * count, dtype=torch.float32, device=self.device)
        native.check(self.lib.sdg_culler_eval(_ptr(self.params), _ptr(self.w1), _ptr(points), self.shapes, count,
                                              _ptr(out), ct.c_void_p(self.stream.cuda_stream)))
        self.stream.synchronize()
        return out

    @_engine_stream
    def surface(self, count, seed):
        """``count`` points on each shape's surface (label 0)."""
        torch = _torch()
        faces = np.cumsum([0] + [len(sh.faces) for sh in self.engine.library.shapes]).astype(np.uint32)
        starts = torch.from_numpy(faces.view(np.int32)).to(self.device)
        triangles = self.engine.buffers["meshTriangles"]
        out = torch.zeros((self.shapes * count, 4), dtype=torch.float32, device=self.device)
        native.check(self.lib.sdg_culler_surface(ct.c_void_p(triangles.ptr()), _ptr(starts), self.shapes, count, seed,
                                                 _ptr(out), ct.c_void_p(self.stream.cuda_stream)))
        self.stream.synchronize()
        return out

    def _root_boxes(self):
        """Each shape's root box (low, high), the frame of its margin cells."""
        g = self.engine.layout.geometry
        roots = g["meshRoots"][:, 0].astype(np.int64)
        return g["meshMin"][roots, :3].astype(np.float32), g["meshMax"][roots, :3].astype(np.float32)

    def _cells(self, points):
        """Margin cell of each (shape-major) point, on the device."""
        torch = _torch()
        low, high = (torch.from_numpy(a).to(self.device) for a in self._root_boxes())
        count = points.shape[0] // self.shapes
        x = points[:, :3].view(self.shapes, count, 3)
        q = (x - low[:, None, :]) / (high - low)[:, None, :]
        k = torch.clamp(torch.floor(q * CELLS), 0, CELLS - 1).to(torch.int64)
        return ((k[..., 2] * CELLS + k[..., 1]) * CELLS + k[..., 0]).reshape(-1)

    @_engine_stream
    def calibrate(self):
        """Margins per shape: the largest run-time prediction at 3 x points fresh
        inside samples (the inside half of a shell sample, the whole interior
        and the surface itself), plus ``slack``; and per cell of an 8^3 grid
        over the shape's root box, the largest at the inside samples of the
        cell and its 26 neighbours, plus ``slack`` (the whole-shape margin
        where those cells hold fewer than ``min_cell_samples``).  A run-time
        node is skipped only above its cell's margin."""
        torch = _torch()
        s = ct.c_void_p(self.stream.cuda_stream)
        native.check(self.lib.sdg_culler_round(_ptr(self.params), _ptr(self.w1), self.shapes, s))
        keys = torch.zeros(self.shapes, dtype=torch.int32, device=self.device)
        cells = self.lib.sdg_culler_margin_cells()
        cell_keys = torch.zeros(self.shapes * cells, dtype=torch.int32, device=self.device)
        cell_counts = torch.zeros(self.shapes * cells, dtype=torch.int32, device=self.device)
        e = self.engine
        geometry = [ct.c_void_p(e.buffers[k].ptr()) for k in ("meshRoots", "meshMin", "meshMax")]
        for seed, kind in ((self.seed + 101, "shell"), (self.seed + 202, "inside"), (self.seed + 303, "surface")):
            if kind == "surface":
                pts = self.surface(self.points, seed)
            else:
                pts = self.sample(self.points, seed, inside_only=kind == "inside")
            pred = self.predict(pts)
            native.check(self.lib.sdg_culler_inside_max(_ptr(pts), _ptr(pred), self.shapes, self.points,
                                                        _ptr(keys), s))
            native.check(self.lib.sdg_culler_inside_max_cells(_ptr(pts), _ptr(pred), self.shapes, self.points,
                                                              *geometry, _ptr(cell_keys), _ptr(cell_counts), s))
            if kind == "shell":
                self.validation = (pts, pred)
        self.stream.synchronize()
        self.margins = _decode(keys.cpu().numpy()) + np.float32(self.slack)
        best = _decode(cell_keys.cpu().numpy()).reshape(self.shapes, CELLS, CELLS, CELLS)
        count = cell_counts.cpu().numpy().astype(np.int64).reshape(self.shapes, CELLS, CELLS, CELLS)
        best = np.where(count > 0, best, -np.inf)
        # Each cell with its 26 neighbours (the grid edge replicated).
        pb = np.pad(best, ((0, 0), (1, 1), (1, 1), (1, 1)), mode="edge")
        pc = np.pad(count, ((0, 0), (1, 1), (1, 1), (1, 1)), mode="edge")
        near = np.full_like(best, -np.inf)
        total = np.zeros_like(count)
        for dz in range(3):
            for dy in range(3):
                for dx in range(3):
                    window = (slice(None), slice(dz, dz + CELLS), slice(dy, dy + CELLS), slice(dx, dx + CELLS))
                    near = np.maximum(near, pb[window])
                    total += pc[window]
        whole = self.margins[:, None, None, None]
        cell = np.where(total >= self.min_cell_samples, np.minimum(near + np.float32(self.slack), whole), whole)
        self.cell_margins = cell.reshape(self.shapes, -1).astype(np.float32)
        return self.margins

    def cull_rate(self):
        """Fraction of validation shell points outside the shape that are culled
        (against their cells' margins)."""
        torch = _torch()
        pts, pred = self.validation
        cells = self._cells(pts).view(self.shapes, -1)
        margin = torch.from_numpy(self.cell_margins).to(self.device).gather(1, cells)
        outside = pts[:, 3].view(self.shapes, -1) > 0
        culled = (pred.view(self.shapes, -1) > margin) & outside
        return float(culled.sum().item() / max(int(outside.sum().item()), 1))

    @_engine_stream
    def attach(self, engine=None):
        """Install parameters, BF16 weights and margins in an engine's buffers."""
        e = engine or self.engine
        if self.margins is None:
            self.calibrate()
        e.buffers["cullerParams"].copy_from_numpy(self.params.cpu().numpy())
        e.buffers["cullerW1"].copy_from_numpy(self.w1.cpu().numpy())
        margins = np.concatenate([self.margins[:, None], self.cell_margins], axis=1).astype(np.float32)
        e.buffers["cullerMargin"].copy_from_numpy(np.ascontiguousarray(margins))
        e.culler = self
        return e

    def detach(self, engine=None):
        (engine or self.engine).culler = None
