"""ctypes wrapper of the calc_deltas oracle (oracle/deltas.c).

TEST INFRASTRUCTURE ONLY (see the package docstring).  ``calc_deltas``
mirrors experiment_scripts/utils.py:46-89 with the open3d raycasting scene
replaced by the exact float32 point-triangle distance stated in deltas.c;
``compute_distance`` is that distance for a batch of points.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "deltas.c")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB = os.path.join(_OUT_DIR, "libdeltas_oracle.so")

_lib = None


def build(force=False):
    """Compile deltas.c with gcc (float32, no contraction, OpenMP threads)."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_SRC) > os.path.getmtime(_LIB):
        tmp = _LIB + f".tmp{os.getpid()}"
        subprocess.check_call([
            "gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
            "-fopenmp", _SRC, "-o", tmp, "-lm"])
        os.replace(tmp, _LIB)
    return _LIB


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        P, I64, F = ctypes.c_void_p, ctypes.c_int64, ctypes.c_float
        lib.mpl_oracle_tri_dist.argtypes = [P, P, P, P]
        lib.mpl_oracle_tri_dist.restype = F
        lib.mpl_oracle_compute_distance.argtypes = [P, P, I64, P, I64, P]
        lib.mpl_oracle_calc_deltas.argtypes = [P, I64, ctypes.c_int, P, I64, P, I64, F, F,
                                               ctypes.c_int, F, F, ctypes.c_int, ctypes.c_int,
                                               P]
        lib.mpl_oracle_calc_deltas.restype = ctypes.c_int
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _mesh(positions, faces):
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    fc = np.ascontiguousarray(faces, np.int32).reshape(-1, 3)
    if fc.size and (fc.min() < 0 or fc.max() >= pos.shape[0]):
        raise ValueError("face index out of range")
    return pos, fc


def tri_dist(p, a, b, c):
    """Distance from p to the triangle (a, b, c), float32."""
    arr = [np.ascontiguousarray(v, np.float32).reshape(3) for v in (p, a, b, c)]
    return float(_load().mpl_oracle_tri_dist(*[_ptr(v) for v in arr]))


def compute_distance(positions, faces, points):
    """Unsigned distance of each point [n, 3] to the triangle mesh (brute
    force), float32; NaN for a point with a non-finite coordinate."""
    pos, fc = _mesh(positions, faces)
    pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
    out = np.empty(pts.shape[0], np.float32)
    _load().mpl_oracle_compute_distance(_ptr(pos), _ptr(fc), fc.shape[0], _ptr(pts),
                                        pts.shape[0], _ptr(out))
    return out


def first_step(max_delta, n_iters):
    """``step_delta = max_delta / n_iters`` of experiment_scripts/utils.py:57,
    as the float32 value the loop starts from: the quotient is taken in
    max_delta's own precision (double for a Python number, float32 for a
    float32 scalar or 0-d array, which is what the trainers pass as a
    tensor) and then rounded to float32."""
    q = np.asarray(max_delta) / n_iters if isinstance(max_delta, (np.ndarray, np.generic)) \
        else float(max_delta) / n_iters
    return float(np.float32(q))


def calc_deltas(vertices, positions, faces, max_delta=0.05, n_iters=100, eps=2e-4, cell=0.0,
                force_iters=None, fast=False, bvh=False):
    """The reference's calc_deltas: returns ([M, C + 1] float32 rows, the
    number of iterations run).  ``cell`` > 0 searches a uniform grid of that
    cell side instead of every triangle (same result).  ``force_iters`` runs
    exactly that many iterations (each vertex's path depends on the others
    only through the stopping point, so a subset of a larger run is checked
    with the larger run's iteration count).  ``fast`` (with ``cell`` > 0)
    decides each step with early exits and bounding-sphere skips instead of
    the minimum (same result).  ``bvh`` decides the same way over a
    bounding-volume hierarchy instead of a grid (``cell`` unused; the timed
    CPU baseline uses it: open3d's scene is a hierarchy too)."""
    V = np.ascontiguousarray(vertices, np.float32)
    M, C = V.shape
    if M == 0:
        raise ValueError("calc_deltas needs at least one vertex (the reference's max of an "
                         "empty tensor raises)")
    pos, fc = _mesh(positions, faces)
    out = np.empty((M, C + 1), np.float32)
    it = _load().mpl_oracle_calc_deltas(_ptr(V), M, C, _ptr(pos), pos.shape[0], _ptr(fc),
                                        fc.shape[0], float(np.float32(max_delta)),
                                        first_step(max_delta, int(n_iters)), int(n_iters),
                                        float(np.float32(eps)), float(cell),
                                        -1 if force_iters is None else int(force_iters),
                                        2 if bvh else (1 if fast else 0), _ptr(out))
    if it < 0:
        raise ValueError("calc_deltas: bad arguments (needs C >= 6 columns and n_iters >= 1)")
    return out, it
