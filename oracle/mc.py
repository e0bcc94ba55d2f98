"""ctypes wrapper of the CPU marching-cubes oracle (oracle/mc.c).

TEST INFRASTRUCTURE ONLY (see the package docstring).  ``marching_cubes``
mirrors the call at i3d/meshing.py:291-313: it returns empty arrays when the
iso level is outside the value range, otherwise vertices shifted by the
origin, faces, normals and values.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "mc.c")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB = os.path.join(_OUT_DIR, "libmc_oracle.so")
_HDR = os.path.join(_HERE, "..", "mplicits_gb300", "csrc", "mc_tables.h")

_lib = None


def build(force=False):
    """Compile mc.c with gcc (float32 without contraction, OpenMP threads)."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    stale = force or not os.path.exists(_LIB) or any(
        os.path.getmtime(s) > os.path.getmtime(_LIB) for s in (_SRC, _HDR))
    if stale:
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
        P = ctypes.c_void_p
        I64 = ctypes.c_int64
        lib.mpl_oracle_mc_count.argtypes = [P, I64, I64, ctypes.c_float, P, P]
        lib.mpl_oracle_mc_emit.argtypes = [P, I64, I64, ctypes.c_float, ctypes.c_float,
                                           P, P, P, P, P, P, P, P, P]
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def marching_cubes_raw(S, iso=0.0, voxel_size=1.0, origin=(0.0, 0.0, 0.0)):
    """Canonical-order marching cubes of a C-order [N, N, N] float32 volume,
    or of a slab [NI, N, N] of NI >= 2 consecutive i-planes of one (vertex
    coordinates then count i from the slab's first plane)."""
    S = np.ascontiguousarray(S, np.float32)
    NI, N = S.shape[0], S.shape[1]
    assert S.shape == (NI, N, N) and NI >= 1
    lib = _load()
    sv = np.zeros(NI, np.int64)
    st = np.zeros(NI, np.int64)
    lib.mpl_oracle_mc_count(_ptr(S), NI, N, ctypes.c_float(iso), _ptr(sv), _ptr(st))
    vbase = np.concatenate([[0], np.cumsum(sv)[:-1]]).astype(np.int64)
    tbase = np.concatenate([[0], np.cumsum(st)[:-1]]).astype(np.int64)
    V, F = int(sv.sum()), int(st.sum())
    verts = np.zeros((V, 3), np.float32)
    normals = np.zeros((V, 3), np.float32)
    values = np.zeros(V, np.float32)
    faces = np.zeros((F, 3), np.int32)
    vmask = np.zeros(NI * N * N, np.uint8)
    vprefix = np.zeros(NI * N * N, np.int64)
    org = np.asarray(origin, np.float32)
    lib.mpl_oracle_mc_emit(_ptr(S), NI, N, ctypes.c_float(iso), ctypes.c_float(voxel_size),
                           _ptr(org), _ptr(vbase), _ptr(tbase), _ptr(vmask), _ptr(vprefix),
                           _ptr(verts), _ptr(normals), _ptr(values), _ptr(faces))
    return verts, faces, normals, values


def marching_cubes(S, voxel_grid_origin, voxel_size, offset=None, scale=None):
    """Restates convert_sdf_samples_to_ply (i3d/meshing.py:267-313)."""
    S = np.asarray(S, np.float32)
    level = 0.0
    if level < S.min() or level > S.max():
        print("Surface level must be within volume data range.")
        return (np.zeros((0, 3)), np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0))
    verts, faces, normals, values = marching_cubes_raw(
        S, level, voxel_size, voxel_grid_origin)
    if scale is not None:
        verts = verts / scale
    if offset is not None:
        verts = verts - offset
    return verts, faces, normals, values
