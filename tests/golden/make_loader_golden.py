"""Golden files of the checkpoint loaders and of the adaptive band widths,
made by the reference's own code.

    python tests/golden/make_loader_golden.py --ref <reference checkout>

(or with ``MPLICITS_REFERENCE`` set to it).  Writes, next to this script:

* ``ref_siren_w64.pth``: ``torch.save`` of the state_dict of the reference's
  ``i3d.model.SIREN(3, 1, [64, 64], w0=30)`` after ``torch.manual_seed(5)``,
  the file a reference user hands to ``from_pth`` (i3d/util.py:79-142);
* ``ref_siren_w64_v1.pth``: the same tensors under the keys of the old SIREN
  class (``net.net.{i}.0.weight|bias``), which ``from_pth`` upgrades;
* ``loaders.npz``: 512 seeded probe points in [-1, 1]^3, the reference
  model's FP32 output on them, and what the reference's
  ``i3d.model.from_pth`` wrote as ``<name>_v2.pth`` for the v1 file (its key
  order and tensors);
* ``adaptive_deltas.npz``: the reference's ``adaptive_deltas``
  (reconstruct.py:18-33) on the tiny three-level model
  (tiny_three_level.npz, w0 = 30) over 10,000 seeded points near its zero
  set, in chunks of 4,096 and of 2^18; ``open3d`` (absent) is stubbed by a
  reader that returns those points, and ``i3d.meshing``'s ``plyfile`` and
  ``skimage`` imports are stubbed;
* ``multistage_increasing.npz``: the reference's create_mesh_multistage
  (i3d/meshing.py:135-264) on the same model with band widths that grow
  from one level to the next (0.005 then 0.05), 24^3 grid, chunks of 37
  points (10 chunks stop after level 0: no point of theirs is in the first
  band): the volume it hands to marching cubes and the points each residual
  level evaluated.  Its CUDA stream synchronisation is shimmed to
  a no-op (the loop runs on the CPU here).
"""

from __future__ import annotations

import os
import shutil
import sys
import tempfile
import types

import numpy as np
import torch

REF = None  # the reference checkout: main() sets it from --ref PATH or MPLICITS_REFERENCE
HERE = os.path.dirname(os.path.abspath(__file__))
_POINTS = {}


def _reference_root():
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from refroot import reference_root
    return reference_root()


def _stub():
    sys.modules["plyfile"] = types.ModuleType("plyfile")
    sk = types.ModuleType("skimage")
    skm = types.ModuleType("skimage.measure")
    skm.marching_cubes = None
    sk.measure = skm
    sys.modules["skimage"] = sk
    sys.modules["skimage.measure"] = skm
    o3d = types.ModuleType("open3d")
    o3d.io = types.SimpleNamespace(
        read_point_cloud=lambda path: types.SimpleNamespace(points=_POINTS[path]))
    sys.modules["open3d"] = o3d
    sys.path.insert(0, REF)


def tiny_reference_models(SIREN):
    d = np.load(os.path.join(HERE, "tiny_three_level.npz"))
    models = []
    for i in range(3):
        m = SIREN(3, 1, [32, 32, 32], w0=30, delay_init=True)
        m.load_state_dict({k[3:]: torch.from_numpy(d[k]) for k in d.files
                           if k.startswith(f"L{i}.")})
        models.append(m.eval())
    return models


def main():
    global REF
    REF = _reference_root()
    _stub()
    from i3d.model import SIREN, from_pth
    import reconstruct as ref_reconstruct

    torch.manual_seed(5)
    model = SIREN(3, 1, [64, 64], w0=30)
    sd = model.state_dict()
    torch.save(sd, os.path.join(HERE, "ref_siren_w64.pth"))
    v1 = type(sd)((f"net.{k}", v.clone()) for k, v in sd.items())
    torch.save(v1, os.path.join(HERE, "ref_siren_w64_v1.pth"))

    rng = np.random.default_rng(17)
    probe = rng.uniform(-1, 1, (512, 3)).astype(np.float32)
    with torch.no_grad():
        out = model(torch.from_numpy(probe))["model_out"].squeeze(-1).numpy()
    tmp = tempfile.mkdtemp(prefix="mplv1")
    try:
        p = os.path.join(tmp, "ref_siren_w64_v1.pth")
        shutil.copy(os.path.join(HERE, "ref_siren_w64_v1.pth"), p)
        loaded = from_pth(p, w0=30)
        v2 = torch.load(os.path.join(tmp, "ref_siren_w64_v1_v2.pth"))
        with torch.no_grad():
            out_v1 = loaded(torch.from_numpy(probe))["model_out"].squeeze(-1).numpy()
    finally:
        shutil.rmtree(tmp)
    arrays = {"probe": probe, "out": out, "out_v1": out_v1,
              "v2_keys": np.array(list(v2.keys()))}
    for k, v in v2.items():
        arrays[f"v2.{k}"] = v.numpy()
    np.savez_compressed(os.path.join(HERE, "loaders.npz"), **arrays)

    # adaptive band widths on points near the tiny model's zero set
    models = tiny_reference_models(SIREN)
    cand = rng.uniform(-1, 1, (200000, 3)).astype(np.float32)
    with torch.no_grad():
        f0 = models[0](torch.from_numpy(cand))["model_out"].squeeze(-1).numpy()
    pts = cand[np.argsort(np.abs(f0))[:10000]]
    pts = pts[rng.permutation(pts.shape[0])]
    _POINTS["cloud.ply"] = pts.astype(np.float64)
    res = {"points": pts}
    for batch in (4096, 2 ** 18):
        res[f"deltas_batch{batch}"] = np.array(
            ref_reconstruct.adaptive_deltas(models, "cloud.ply", "cpu", batch=batch), np.float64)
    np.savez_compressed(os.path.join(HERE, "adaptive_deltas.npz"), **res)

    # band widths that grow: masks over whole chunks and the per-chunk break
    from i3d import meshing
    evaluated = [[] for _ in models]
    captured = {}

    class Rec(torch.nn.Module):
        def __init__(self, m, i):
            super().__init__()
            self.m, self.i = m, i

        def forward(self, x):
            evaluated[self.i].append(x.detach().clone())
            return self.m(x)

    class NoSync:
        def synchronize(self):
            return None

    orig_stream, orig_conv = torch.cuda.current_stream, meshing.convert_sdf_samples_to_ply

    def conv(vol, *a, **k):
        captured["volume"] = np.array(vol, copy=True)
        return np.zeros((0, 3)), np.zeros((0, 3), np.int64), np.zeros((0, 3)), np.zeros(0)

    torch.cuda.current_stream = lambda *a, **k: NoSync()
    meshing.convert_sdf_samples_to_ply = conv
    N, deltas, chunk = 24, [0.005, 0.05], 37  # 10 of 374 chunks break after level 0
    try:
        meshing.create_mesh_multistage([Rec(m, i) for i, m in enumerate(models)], deltas=deltas,
                                       N=N, max_batch=chunk, device="cpu", silent=True)
    finally:
        torch.cuda.current_stream = orig_stream
        meshing.convert_sdf_samples_to_ply = orig_conv
    inc = {"N": np.array(N), "deltas": np.array(deltas), "chunk": np.array(chunk),
           "S": captured["volume"].reshape(-1)}
    for i in (1, 2):
        inc[f"band{i}_pts"] = torch.cat(evaluated[i]).numpy() if evaluated[i] else \
            np.zeros((0, 3), np.float32)
    np.savez_compressed(os.path.join(HERE, "multistage_increasing.npz"), **inc)
    print("increasing bands: evaluated", [inc[f"band{i}_pts"].shape[0] for i in (1, 2)])
    print("loaders:", out[:3], "adaptive deltas:", res["deltas_batch4096"],
          res["deltas_batch262144"])


if __name__ == "__main__":
    main()
