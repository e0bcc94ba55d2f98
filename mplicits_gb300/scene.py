"""Triangle scene and the tubular-neighbourhood deltas on the GPU.

The neighbourhood trainers build an open3d ``RaycastingScene`` from the
mesh (experiment_scripts/train_sdf_on_neighborhood.py:145-146) and hand it
to ``calc_deltas`` (experiment_scripts/utils.py:46-89), which bisects, per
vertex, the radius of the largest ball along the normal that touches the
mesh only at the vertex.  ``RaycastingScene`` here is a uniform grid over
the triangles built by libmplicits (no open3d), with the same
``add_triangles`` / ``compute_distance`` calls; ``calc_deltas`` takes the
same arguments as the reference's and runs every iteration on the device.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi


class RaycastingScene:
    """Nearest-triangle distance queries over one triangle mesh.

    ``add_triangles(positions, faces)`` (or the constructor's arguments)
    takes positions [V, 3] and integer faces [F, 3] (tensors or arrays);
    a second call replaces the mesh.  ``cell`` is the grid's cell side
    (default: twice the mean edge length).

    Building and releasing a scene synchronise: a replaced or collected
    scene's memory is freed after a device-wide synchronisation.  Keep a
    scene alive (and call no ``add_triangles``) while any stream of the
    process is capturing a CUDA graph; that synchronisation would end the
    capture with an error.
    """

    def __init__(self, positions=None, faces=None, device="cuda", cell=0.0):
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise RuntimeError("mplicits_gb300 builds triangle scenes on a CUDA device only")
        self.cell = float(cell)
        self._handle = None
        if positions is not None:
            self.add_triangles(positions, faces)

    def add_triangles(self, positions, faces):
        pos = torch.as_tensor(positions).to(self.device, torch.float32).reshape(-1, 3).contiguous()
        fc = torch.as_tensor(faces).to(self.device, torch.int32).reshape(-1, 3).contiguous()
        self._release()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            capi.check(capi.load().mpl_scene_create(
                capi.ptr(pos), pos.shape[0], capi.ptr(fc), fc.shape[0], self.cell,
                ctypes.byref(h), capi.stream_ptr()), "mpl_scene_create")
        self._handle = h
        self.n_faces = fc.shape[0]
        return 0

    def info(self):
        """Grid geometry: lower corner, cell side, cells per axis, entries."""
        lo = (ctypes.c_float * 3)()
        cell = ctypes.c_float()
        dims = (ctypes.c_int32 * 3)()
        refs = ctypes.c_int64()
        capi.check(capi.load().mpl_scene_info(self.handle, lo, ctypes.byref(cell), dims,
                                              ctypes.byref(refs)), "mpl_scene_info")
        return {"lo": list(lo), "cell": cell.value, "dims": list(dims), "entries": refs.value}

    @property
    def handle(self):
        if self._handle is None:
            raise RuntimeError("the scene has no triangles: call add_triangles first")
        return self._handle

    def compute_distance(self, points):
        """Unsigned distance of each point [n, 3] to the mesh (float32 [n])."""
        p = torch.as_tensor(points).to(self.device, torch.float32).reshape(-1, 3).contiguous()
        out = torch.empty(p.shape[0], dtype=torch.float32, device=self.device)
        with torch.cuda.device(self.device):
            capi.check(capi.load().mpl_scene_compute_distance(
                self.handle, capi.ptr(p), p.shape[0], capi.ptr(out), capi.stream_ptr()),
                "mpl_scene_compute_distance")
        return out

    def _release(self):
        if self._handle is not None:
            with torch.cuda.device(self.device):
                capi.load().mpl_scene_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self._release()
        except Exception:  # interpreter shutdown: the library may be gone
            pass


def first_step(max_delta, n_iters):
    """float32 first step of calc_deltas, ``max_delta / n_iters``
    (experiment_scripts/utils.py:57): a tensor divides in its own dtype, a
    Python number in double; the loop then holds it as float32."""
    if isinstance(max_delta, torch.Tensor):
        return float((max_delta.detach().cpu() / n_iters).to(torch.float32).item())
    if isinstance(max_delta, (np.ndarray, np.generic)):
        return float(np.float32(np.asarray(max_delta) / n_iters))
    return float(np.float32(float(max_delta) / n_iters))


def calc_deltas(vertices, scene, max_delta=0.05, n_iters=100, device=None, eps=2e-4,
                return_iterations=False):
    """Drop-in for experiment_scripts/utils.py:46-89.

    ``vertices`` [M, C >= 6] (xyz, normal, ...); returns [M, C + 1] on the
    scene's device: the rows with unit normals and the neighbourhood radius
    appended.  ``max_delta`` may be a Python number or a 0-d tensor (the
    reference's callers pass ``max |f(v)|`` as a tensor); the loop compares
    against it in float32, and the first step is ``max_delta / n_iters``
    taken in max_delta's own precision (double for a Python number, float32
    for a float32 tensor) and rounded to float32, as utils.py:57 does (a
    device tensor is read on the host once).  With ``return_iterations``
    also returns the number of iterations run (one more host read).  The
    iterations themselves run without host round trips.
    """
    dev = scene.device if device is None else torch.device(device)
    if dev.type != "cuda" or (dev.index if dev.index is not None else torch.cuda.current_device()) \
            != (scene.device.index if scene.device.index is not None
                else torch.cuda.current_device()):
        raise ValueError(f"calc_deltas runs on the scene's device ({scene.device}), not {dev}")
    V = torch.as_tensor(vertices).detach().to(dev, torch.float32).contiguous()
    if V.dim() != 2 or V.shape[1] < 6:
        raise ValueError("calc_deltas needs vertices [M, >= 6] (xyz, normal, ...)")
    M, C = V.shape
    if M == 0:
        raise ValueError("calc_deltas needs at least one vertex (the reference's max of an "
                         "empty tensor raises)")
    if int(n_iters) < 1:
        raise ValueError("n_iters must be >= 1")
    md = float(torch.as_tensor(max_delta, dtype=torch.float32).item())
    step0 = first_step(max_delta, int(n_iters))
    nbytes = ctypes.c_int64()
    lib = capi.load()
    capi.check(lib.mpl_calc_deltas_scratch_bytes(M, int(n_iters), ctypes.byref(nbytes)),
               "mpl_calc_deltas_scratch_bytes")
    scratch = torch.empty(nbytes.value, dtype=torch.uint8, device=dev)
    out = torch.empty(M, C + 1, dtype=torch.float32, device=dev)
    iters = torch.zeros(1, dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        capi.check(lib.mpl_calc_deltas(scene.handle, capi.ptr(V), M, C, md, step0, int(n_iters),
                                       float(eps), capi.ptr(scratch), capi.ptr(out),
                                       capi.ptr(iters), capi.stream_ptr()), "mpl_calc_deltas")
    if return_iterations:
        return out, int(iters.item())
    return out
