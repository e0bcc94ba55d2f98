"""Golden vectors of the residual trainers' batch construction.

    python tests/golden/make_train_batch.py --ref <reference checkout>

Runs the reference's own ``create_training_data_on_neighborhood``
(experiment_scripts/utils.py:92-169) from a reference checkout
(``--ref`` or ``MPLICITS_REFERENCE``) on a small seeded vertex array, with and without the
neighbourhood delta column and dithering.  ``open3d`` and ``plyfile`` are
imported at module level there but not used by this function, so both are
stubbed.  The random draws the function makes (``torch.randperm`` for the
sample, ``torch.rand`` for the offsets) are recovered by replaying the
generator from the same seed, so the fixture holds the inputs the GPU
kernel is given (indices, uniforms) next to the reference's outputs.
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


def _stub():
    o3d = types.ModuleType("open3d")
    o3c = types.ModuleType("open3d.core")
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


def main():
    global REF
    REF = _reference_root()
    _stub()
    from utils import create_training_data_on_neighborhood  # the reference module

    rng = np.random.default_rng(17)
    M = 300
    xyz = rng.uniform(-0.7, 0.7, (M, 3)).astype(np.float32)
    nrm = xyz / np.linalg.norm(xyz, axis=1, keepdims=True)
    dn = rng.uniform(1e-4, 3e-3, (M, 1)).astype(np.float32)
    verts = np.concatenate([xyz, nrm.astype(np.float32), dn], axis=1)
    out = {"vertices": verts}
    cases = [(96, 0.01, False, True), (96, 0.02, True, True), (64, 0.01, False, False),
             (M, 0.01, True, True)]
    for c, (n, delta, neigh, dither) in enumerate(cases):
        seed = 1000 + c
        torch.manual_seed(seed)
        res = create_training_data_on_neighborhood(torch.from_numpy(verts), n, delta=delta,
                                                   use_neigh_delta=neigh,
                                                   dithering_sampling=dither)
        pts, normals, sdfs = res["on_surf"]
        # replay the draws of sample_on_surface and the offsets
        torch.manual_seed(seed)
        if n == M:
            idx = torch.arange(M)
        else:
            idx = torch.randperm(M)[:n]
        u = torch.rand((min(n, M), 3))
        out.update({f"c{c}.n": np.array(n), f"c{c}.delta": np.array(delta),
                    f"c{c}.neigh": np.array(neigh), f"c{c}.dither": np.array(dither),
                    f"c{c}.idx": idx.numpy().astype(np.int64), f"c{c}.u": u.numpy(),
                    f"c{c}.pts": pts.numpy(), f"c{c}.normals": normals.numpy(),
                    f"c{c}.sdf": sdfs.numpy()})
    np.savez_compressed(os.path.join(HERE, "train_batch.npz"), **out)
    print("written", os.path.join(HERE, "train_batch.npz"))


if __name__ == "__main__":
    main()
