"""Build and load the sm_103a CUDA library behind the C ABI.

The library is plain ``nvcc`` output (``_lib/libsanddem_gb300.so``) loaded with
ctypes; no torch types cross the boundary.  Loading fails loudly when the
library is missing or when no CUDA device is present: there is no CPU
fallback for the step.
"""

import ctypes as ct
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
CSRC = PACKAGE / "csrc"
LIBDIR = PACKAGE / "_lib"
LIBRARY = LIBDIR / "libsanddem_gb300.so"
SOURCES = ("kernels_state.cu", "kernels_contacts.cu", "capi.cu", "culler.cu", "scan_static.cu", "trees.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false keeps the reference's FP32 operation order (no contraction);
# division and square root stay IEEE (no fast math).
FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC"]


def nvcc():
    root = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = Path(root) / "bin" / "nvcc"
    return str(path) if path.exists() else "nvcc"


def build(force=False, verbose=False):
    """Compile every translation unit in parallel and link the shared library."""
    LIBDIR.mkdir(exist_ok=True)
    headers = max(p.stat().st_mtime for p in [*CSRC.glob("*.h"), *CSRC.glob("*.cuh")])
    objects = []
    jobs = []
    for name in SOURCES:
        src = CSRC / name
        obj = LIBDIR / (Path(name).stem + ".o")
        objects.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, headers):
            jobs.append([nvcc(), *ARCH, *FLAGS, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        result = subprocess.run(cmd, capture_output=True, text=True)
        if result.returncode:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{result.stderr}")
        if verbose:
            print(result.stderr)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        list(pool.map(run, jobs))
    if jobs or force or not LIBRARY.exists():
        run([nvcc(), *ARCH, "-shared", "-o", str(LIBRARY), *map(str, objects), "-lcudart"])
    return LIBRARY


_LIB = None


def load():
    """The loaded library; raises if it is missing (build() first)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not LIBRARY.exists():
        raise RuntimeError(
            f"GB300 CUDA library not built ({LIBRARY}); run sand_atlas_dem_gb300.native.build()"
        )
    lib = ct.CDLL(str(LIBRARY))
    P = ct.POINTER
    lib.sdg_abi_version.restype = ct.c_int
    lib.sdg_buffer_count.restype = ct.c_int
    lib.sdg_value_count.restype = ct.c_int
    lib.sdg_last_error.restype = ct.c_char_p
    lib.sdg_dispatch.argtypes = [ct.c_char_p, ct.c_uint32, P(ct.c_void_p), P(ct.c_uint64), P(ct.c_double),
                                 ct.c_uint32, ct.c_void_p]
    lib.sdg_dispatch.restype = ct.c_int
    lib.sdg_reduce_rows.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_uint32, ct.c_uint32, ct.c_int32, ct.c_void_p]
    lib.sdg_reduce_rows.restype = ct.c_int
    lib.sdg_reduce_wall_rows.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_uint32, ct.c_uint32, ct.c_void_p]
    lib.sdg_reduce_wall_rows.restype = ct.c_int
    lib.sdg_engine_create.restype = ct.c_void_p
    lib.sdg_engine_destroy.argtypes = [ct.c_void_p]
    lib.sdg_engine_advance.argtypes = [ct.c_void_p, P(ct.c_void_p), P(ct.c_uint64), P(ct.c_double), ct.c_uint32,
                                       ct.c_uint32, ct.c_uint32, ct.c_void_p]
    lib.sdg_engine_advance.restype = ct.c_int
    lib.sdg_engine_profile.argtypes = [ct.c_void_p, P(ct.c_void_p), P(ct.c_uint64), P(ct.c_double), ct.c_uint32,
                                       P(ct.c_float), ct.c_void_p]
    lib.sdg_engine_profile.restype = ct.c_int
    lib.sdg_exclusive_scan.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_uint32, ct.c_void_p, ct.c_void_p,
                                       ct.c_void_p]
    lib.sdg_exclusive_scan.restype = ct.c_int
    lib.sdg_scan_partials.restype = ct.c_int
    lib.sdg_engine_diagnostics.argtypes = [P(ct.c_void_p), P(ct.c_uint64), P(ct.c_double), ct.c_uint32,
                                           ct.c_void_p, ct.c_void_p, ct.c_uint64, ct.c_void_p, ct.c_void_p]
    lib.sdg_engine_diagnostics.restype = ct.c_int
    lib.sdg_copy_buffers.argtypes = [P(ct.c_void_p), P(ct.c_void_p), P(ct.c_uint64), ct.c_uint32, ct.c_void_p]
    lib.sdg_copy_buffers.restype = ct.c_int
    lib.sdg_exclusive_scan_static.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_uint32, ct.c_void_p, ct.c_void_p]
    lib.sdg_exclusive_scan_static.restype = ct.c_int
    V = ct.c_void_p
    U = ct.c_uint32
    F = ct.c_float
    culler = {
        "sdg_culler_param_count": [],
        "sdg_culler_margin_cells": [],
        "sdg_culler_sample": [P(V), P(ct.c_uint64), P(ct.c_double), U, U, U, U, F, U, V, V, V],
        "sdg_culler_compact": [V, V, V, U, U, U, V, V],
        "sdg_culler_surface": [V, V, U, U, U, V, V],
        "sdg_culler_train_step": [V, V, U, U, U, U, U, F, F, F, V, V, V, V, V, V],
        "sdg_culler_gradients": [V, V, U, U, U, U, U, F, F, V, V, V],
        "sdg_culler_round": [V, V, U, V],
        "sdg_culler_eval": [V, V, V, U, U, V, V],
        "sdg_culler_tile_eval": [V, V, V, U, U, V, V],
        "sdg_culler_inside_max": [V, V, U, U, V, V],
        "sdg_culler_inside_max_cells": [V, V, U, U, V, V, V, V, V, V],
    }
    for name, args in culler.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ct.c_int
    lib.sdg_median_tree_nodes.argtypes = [U, U]
    lib.sdg_median_tree_nodes.restype = U
    lib.sdg_median_trees_scratch.argtypes = [V, U, U]
    lib.sdg_median_trees_scratch.restype = ct.c_uint64
    lib.sdg_median_trees.argtypes = [V, V, V, V, U, U, V, V, V, V, V, ct.c_uint64, V]
    lib.sdg_median_trees.restype = ct.c_int
    lib.sdg_engine_kernels_per_step.argtypes = [ct.c_void_p]
    lib.sdg_engine_kernels_per_step.restype = ct.c_int
    lib.sdg_engine_branch_kernels.argtypes = [ct.c_void_p, ct.c_int]
    lib.sdg_engine_branch_kernels.restype = ct.c_int
    _LIB = lib
    return lib


def check(rc):
    if rc:
        raise RuntimeError("GB300 library call failed: " + load().sdg_last_error().decode())


EXPORTS = (
    "sdg_abi_version",
    "sdg_buffer_count",
    "sdg_value_count",
    "sdg_last_error",
    "sdg_dispatch",
    "sdg_reduce_rows",
    "sdg_reduce_wall_rows",
    "sdg_engine_create",
    "sdg_engine_destroy",
    "sdg_engine_advance",
    "sdg_engine_profile",
    "sdg_engine_diagnostics",
    "sdg_engine_kernels_per_step",
    "sdg_engine_branch_kernels",
    "sdg_exclusive_scan",
    "sdg_scan_partials",
    "sdg_copy_buffers",
    "sdg_exclusive_scan_static",
    "sdg_culler_param_count",
    "sdg_culler_sample",
    "sdg_culler_surface",
    "sdg_culler_compact",
    "sdg_culler_train_step",
    "sdg_culler_gradients",
    "sdg_culler_round",
    "sdg_culler_eval",
    "sdg_culler_tile_eval",
    "sdg_culler_inside_max",
    "sdg_culler_inside_max_cells",
    "sdg_culler_margin_cells",
    "sdg_median_tree_nodes",
    "sdg_median_trees_scratch",
    "sdg_median_trees",
)
PHASES = ("drift", "neighbours", "pair_cull", "node_filter", "node_query", "contact_emit", "friction_and_history",
          "force_reduction", "final_kick")
