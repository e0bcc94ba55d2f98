"""Generate the golden vectors that pin the oracle to the reference.

Run where a reference checkout is at hand:

    python tests/golden/make_golden.py --ref <reference checkout>

(or with ``MPLICITS_REFERENCE`` set to it).

It imports the reference's own ``i3d`` package.  ``i3d.meshing`` imports
``plyfile`` and ``skimage`` at module level; neither is installed, so both are
stubbed: the ``marching_cubes`` stub only records the volume it is handed.
``create_mesh_multistage`` synchronises the CUDA stream unconditionally
(i3d/meshing.py:219,238), which raises without a GPU, so that call is shimmed
to a no-op while the reference loop runs on the CPU.  Outputs (small ``.npz``
files) land next to this script.
"""

from __future__ import annotations

import hashlib
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

captured = {}


def _install_stubs():
    sys.modules["plyfile"] = types.ModuleType("plyfile")
    sk = types.ModuleType("skimage")
    skm = types.ModuleType("skimage.measure")

    def marching_cubes(vol, level, spacing=None):
        captured["volume"] = np.array(vol, copy=True)
        z = np.zeros((0, 3))
        return z, z.astype(np.int64), z, np.zeros(0)

    skm.marching_cubes = marching_cubes
    sk.measure = skm
    sys.modules["skimage"] = sk
    sys.modules["skimage.measure"] = skm
    sys.path.insert(0, REF)


class _NoSync:
    def synchronize(self):
        return None


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def state_dict_np(model):
    return {k: v.detach().cpu().numpy().astype(np.float32) for k, v in model.state_dict().items()}


def main():
    global REF
    REF = _reference_root()
    _install_stubs()
    from i3d.model import SIREN
    from i3d import meshing, diff_operators
    from i3d.loss_functions import loss_add_detail_fine

    torch.set_num_threads(max(1, os.cpu_count() or 1))

    # ---- grid coordinates (i3d/meshing.py:11-69) ----------------------------
    grid = {}
    for N in (2, 3, 4, 5, 16, 127, 128, 512):
        g = meshing.gen_mc_coordinate_grid(N, 2.0 / (N - 1))[:, :3].numpy()
        grid[f"sha_{N}"] = np.array(sha(g))
        sel = np.unique(np.linspace(0, N ** 3 - 1, 257).astype(np.int64))
        grid[f"idx_{N}"] = sel
        grid[f"xyz_{N}"] = g[sel]
        del g
    np.savez_compressed(os.path.join(HERE, "grid.npz"), **grid)

    # ---- config-1 SIREN (seed 0) probe outputs (i3d/model.py:76-129) --------
    torch.manual_seed(0)
    m1 = SIREN(3, 1, [256, 256, 256], w0=30)
    sd = state_dict_np(m1)
    g16 = meshing.gen_mc_coordinate_grid(16, 2.0 / 15)[:, :3]
    rng = np.random.default_rng(7)
    xr = torch.from_numpy(rng.uniform(-1, 1, (1024, 3)).astype(np.float32))
    with torch.no_grad():
        y16 = m1(g16)["model_out"].squeeze(-1).numpy()
        yr = m1(xr)["model_out"].squeeze(-1).numpy()
    # gradient through the reference autograd path (i3d/diff_operators.py:259)
    out = m1(xr[:256])
    gr = diff_operators.gradient(out["model_out"], out["model_in"]).detach().numpy()
    probe = {f"sha_{k}": np.array(sha(v)) for k, v in sd.items()}
    probe.update(x16=g16.numpy(), y16=y16, xr=xr.numpy(), yr=yr, grad_r=gr)
    np.savez_compressed(os.path.join(HERE, "siren_cfg1_probe.npz"), **probe)

    # ---- tiny three-level model: full weights + band-culled loop ------------
    levels = []
    for seed in (11, 12, 13):
        torch.manual_seed(seed)
        levels.append(SIREN(3, 1, [32, 32, 32], w0=30))
    # scale the residual levels down so they act as residuals
    with torch.no_grad():
        for lv, s in zip(levels[1:], (0.1, 0.02)):
            lv.net[-1][0].weight.mul_(s)
            lv.net[-1][0].bias.mul_(s)
        # move the coarse zero level inside the box
        levels[0].net[-1][0].bias.add_(0.13)
    evaluated = [[] for _ in levels]

    class Rec(torch.nn.Module):
        def __init__(self, m, i):
            super().__init__()
            self.m, self.i = m, i

        def forward(self, x):
            evaluated[self.i].append(x.detach().clone())
            return self.m(x)

    N, deltas = 24, [0.05, 0.02]
    orig = torch.cuda.current_stream
    torch.cuda.current_stream = lambda *a, **k: _NoSync()
    orig_conv = meshing.convert_sdf_samples_to_ply

    def conv(vol, *a, **k):
        captured["volume"] = np.array(vol, copy=True)
        return orig_conv(vol, *a, **k)

    meshing.convert_sdf_samples_to_ply = conv
    try:
        meshing.create_mesh_multistage([Rec(m, i) for i, m in enumerate(levels)], deltas=deltas,
                                       N=N, max_batch=32 ** 3 // 8, device="cpu", silent=True)
        vol_banded = captured["volume"].reshape(-1)
        meshing.create_mesh_multistage(levels, deltas=[], N=N, max_batch=32 ** 3 // 8,
                                       device="cpu", silent=True)
        vol_full = captured["volume"].reshape(-1)
    finally:
        torch.cuda.current_stream = orig
        meshing.convert_sdf_samples_to_ply = orig_conv
    tiny = {}
    for i, lv in enumerate(levels):
        for k, v in state_dict_np(lv).items():
            tiny[f"L{i}.{k}"] = v
    tiny.update(N=np.array(N), deltas=np.array(deltas), S_banded=vol_banded, S_full=vol_full)
    for i in (1, 2):
        pts = torch.cat(evaluated[i]).numpy() if evaluated[i] else np.zeros((0, 3), np.float32)
        tiny[f"band{i}_pts"] = pts
    np.savez_compressed(os.path.join(HERE, "tiny_three_level.npz"), **tiny)

    # ---- the band test at i3d/meshing.py:223 compares in float32 ------------
    d = 0.06  # float32(0.06) < 0.06, so S == float32(0.06) is the edge case
    f = np.float32(d)
    S = np.array([f, np.nextafter(f, np.float32(0)), np.nextafter(f, np.float32(1)),
                  -f, 0.0, np.float32(0.0599999), -np.nextafter(f, np.float32(0))], np.float32)
    mask = (torch.abs(torch.from_numpy(S)) < d).numpy()
    np.savez_compressed(os.path.join(HERE, "band_compare.npz"), S=S, delta=np.array(d), mask=mask)

    # ---- residual loss of the fine trainer (i3d/loss_functions.py:347-394) --
    torch.manual_seed(21)
    fine = SIREN(3, 1, [32, 32, 32], w0=30)
    xb = torch.from_numpy(rng.uniform(-0.8, 0.8, (96, 3)).astype(np.float32))
    nb = torch.nn.functional.normalize(xb, dim=-1)
    gsdf = torch.zeros(96, 1)
    gsdf[32:64, 0] = 0.01
    gsdf[64:, 0] = -1
    loss_fn = loss_add_detail_fine(levels[0], levels[1])
    y = fine(xb)
    losses = loss_fn(y, {"sdf": gsdf, "normals": nb})
    total = sum(losses.values())
    total.backward()
    lf = {f"fine.{k}": v for k, v in state_dict_np(fine).items()}
    lf.update({f"grad.{k}": p.grad.numpy().copy() for k, p in fine.named_parameters()})
    lf.update({f"loss.{k}": np.array(float(v)) for k, v in losses.items()})
    lf.update(x=xb.numpy(), normals=nb.numpy(), sdf=gsdf.numpy())
    np.savez_compressed(os.path.join(HERE, "loss_fine.npz"), **lf)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
