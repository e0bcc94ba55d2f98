"""Golden vectors of the tubular-neighbourhood deltas (calc_deltas).

    python tests/golden/make_calc_deltas.py --ref <reference checkout>

Runs the reference's own ``calc_deltas`` (experiment_scripts/utils.py:46-89)
from a reference checkout (``--ref`` or ``MPLICITS_REFERENCE``).  Its scene is an
open3d ``RaycastingScene`` (open3d 0.19.0, not installed); here a stand-in
object answers ``compute_distance`` with the oracle's float32 point-triangle
distance (oracle/deltas.c, brute force over all triangles) and counts its
calls, which is the number of loop iterations.  ``open3d`` and ``plyfile``
are stubbed at import.  torch's CPU ``sqrt`` (a vectorised kernel) is not
correctly rounded in near-tie cases, while the reference runs on CUDA where
``sqrtf`` is; during the call ``torch.sqrt`` of float32 is replaced by the
correctly rounded one (through float64).  The fixture therefore pins the
oracle's loop (step halving, the two branches, the stopping rule, normal
normalisation, the appended column) to the reference's code; the distance
itself is pinned in tests/test_deltas_oracle.py against float64 geometry.
"""

from __future__ import annotations

import os
import sys
import types

import numpy as np
import torch

REF = None  # the reference checkout: main() sets it from --ref PATH or MPLICITS_REFERENCE


def _reference_root():
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from refroot import reference_root
    return reference_root()
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


class _Tensor:
    def __init__(self, a, dtype=None):
        self.a = np.ascontiguousarray(a, np.float32)

    def numpy(self):
        return self.a


def _stub():
    o3d = types.ModuleType("open3d")
    o3c = types.ModuleType("open3d.core")
    o3c.Tensor = _Tensor
    o3c.Dtype = types.SimpleNamespace(Float32="Float32")
    o3t = types.ModuleType("open3d.t")
    o3g = types.ModuleType("open3d.t.geometry")
    o3g.RaycastingScene = object
    o3t.geometry = o3g
    o3d.t = o3t
    o3d.core = o3c
    sys.modules.update({"open3d": o3d, "open3d.core": o3c, "open3d.t": o3t,
                        "open3d.t.geometry": o3g})
    ply = types.ModuleType("plyfile")
    ply.PlyData = object
    sys.modules["plyfile"] = ply
    sys.path.insert(0, os.path.join(REF, "experiment_scripts"))
    sys.path.insert(0, ROOT)


class Scene:
    """compute_distance of the oracle, counting calls."""

    def __init__(self, positions, faces):
        self.pos, self.faces, self.calls = positions, faces, 0

    def compute_distance(self, pts):
        from oracle import deltas
        self.calls += 1
        return _Tensor(deltas.compute_distance(self.pos, self.faces, pts.numpy()))


def slab(n=8, gap=0.1):
    """Two parallel n x n grids of squares at z = 0 and z = gap, each split
    into triangles; normals point into the gap (+z below, -z above)."""
    u = np.linspace(-0.5, 0.5, n + 1, dtype=np.float32)
    X, Y = np.meshgrid(u, u, indexing="ij")
    sheet = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size, np.float32)], 1)
    top = sheet.copy()
    top[:, 2] = gap
    pos = np.concatenate([sheet, top]).astype(np.float32)
    nrm = np.concatenate([np.tile([0, 0, 1], (sheet.shape[0], 1)),
                          np.tile([0, 0, -1], (sheet.shape[0], 1))]).astype(np.float32)
    faces = []
    for off in (0, sheet.shape[0]):
        for i in range(n):
            for j in range(n):
                a = off + i * (n + 1) + j
                faces += [(a, a + n + 1, a + 1), (a + 1, a + n + 1, a + n + 2)]
    return pos, nrm, np.asarray(faces, np.int32)


def cases():
    from mplicits_gb300 import synthetic
    rng = np.random.default_rng(29)
    pos, nrm, faces = synthetic.surface_mesh(14, 20)
    V = np.concatenate([pos, nrm], 1)
    out = []
    out.append(("sphere", V, pos, faces, 0.05, 100))
    # non-unit normals, one zero normal (NaN displacement), a 7th column
    Vs = V.copy()
    Vs[:, 3:6] *= rng.uniform(0.3, 3.0, (V.shape[0], 1)).astype(np.float32)
    Vs[5, 3:6] = 0.0
    Vs = np.concatenate([Vs, rng.uniform(0, 1e-3, (V.shape[0], 1)).astype(np.float32)], 1)
    out.append(("scaled_normals_extra_column", Vs, pos, faces, 0.08, 100))
    # a few iterations only; a large radius
    out.append(("short_loop", V, pos, faces, 0.3, 7))
    # two facing sheets: the bisection converges to half the gap
    sp, sn, sf = slab()
    Vslab = np.concatenate([sp, sn], 1)
    out.append(("slab", Vslab, sp, sf, 0.2, 100))
    # a vertex on no triangle, far away: its distance exceeds delta + eps
    Viso = np.concatenate([Vslab, np.array([[3.0, 3.0, 3.0, 0, 0, 1]], np.float32)])
    out.append(("isolated_vertex", Viso, sp, sf, 0.2, 60))
    # max_delta as a Python float: the first step is a double quotient
    # rounded to float32, one ulp away from the float32 quotient for these
    out.append(("float_max_delta", V, pos, faces, 0.03, 100))
    out.append(("float_max_delta_1000", V, pos, faces, 0.1, 1000))
    return out


# cases whose max_delta is passed as a Python float (the rest as a 0-d
# float32 tensor, as the reference's trainers do)
FLOAT_CASES = {"float_max_delta", "float_max_delta_1000"}


def main():
    global REF
    REF = _reference_root()
    _stub()
    from utils import calc_deltas  # the reference module

    sqrt = torch.sqrt
    torch.sqrt = lambda x: sqrt(x.double()).float() if x.dtype == torch.float32 else sqrt(x)

    arrays = {}
    names = []
    for name, V, pos, faces, max_delta, n_iters in cases():
        scene = Scene(pos, faces)
        # the reference's trainers pass max_delta as a 0-d float32 tensor
        md = max_delta if name in FLOAT_CASES else torch.tensor(max_delta, dtype=torch.float32)
        res = calc_deltas(torch.from_numpy(V.copy()), scene, max_delta=md, n_iters=n_iters,
                          device=torch.device("cpu"))
        names.append(name)
        arrays[f"{name}__vertices"] = V
        arrays[f"{name}__positions"] = pos
        arrays[f"{name}__faces"] = faces
        arrays[f"{name}__max_delta"] = np.float64(max_delta) if name in FLOAT_CASES \
            else np.float32(max_delta)
        arrays[f"{name}__max_delta_kind"] = np.array("float" if name in FLOAT_CASES else "tensor")
        arrays[f"{name}__n_iters"] = np.int32(n_iters)
        arrays[f"{name}__out"] = res.numpy().astype(np.float32)
        arrays[f"{name}__iterations"] = np.int32(scene.calls)
        d = res.numpy()[:, -1]
        print(f"{name}: {V.shape[0]} vertices, {faces.shape[0]} faces, {scene.calls} iterations, "
              f"delta range {d.min():.5f}..{d.max():.5f}")
    arrays["cases"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "calc_deltas.npz"), **arrays)


if __name__ == "__main__":
    main()
