"""Train the three-level residual model of the 512^3 band-culled workload
with this project's own trainers on the GPU.

    python tests/golden/make_three_level_model.py [--steps 4000 2000 2000] [--out PATH]

Each level is 3 -> 256 x 3 -> 1 with omega0 = 30.  The data is the synthetic
surface of ``mplicits_gb300.synthetic``: 2^18 surface points with their
analytic normals and Gaussian position noise sigma = 0.002 (seed 1), and a
pool of 2^21 uniform points of [-1, 1]^3 with their signed distance.  The
training is ``mplicits_gb300.pipeline.train_three_levels``, the reference
trainers' three stages on the hand-written kernels (forward, loss, double
backward and Adam, lr 1e-4, FP32 master weights, BF16 tensor-core
arithmetic, best-loss state after 10 % warm-up kept):

  coarse  train_sdf.py:238-269 with ``true_sdf`` (i3d/loss_functions.py:
          123-163): surface points (sdf 0, normals) and pool points with
          their signed distance;
  medium  experiment_scripts/train_sdf_on_neighborhood.py with
          ``loss_add_detail``, the coarse level frozen, band delta0 = 0.05;
  fine    train_sdf_on_neighborhood_fine.py with ``loss_add_detail_fine``,
          both coarser levels frozen, band delta1 = 0.01;

the residual batches built as create_training_data_on_neighborhood does
(experiment_scripts/utils.py:92-169), 2^16 surface samples per step.
Output: three_level_sphere.npz (``L{i}.net.{j}.0.weight|bias``, omega not
baked).  Needs a CUDA device.
"""

from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    from mplicits_gb300 import build
    from mplicits_gb300.pipeline import train_three_levels
    from mplicits_gb300.synthetic import SignedDistance, surface_points
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, nargs=3, default=[4000, 2000, 2000])
    ap.add_argument("--batch", type=int, default=1 << 16)
    ap.add_argument("--out", default=os.path.join(HERE, "three_level_sphere.npz"))
    args = ap.parse_args()
    build.build()
    rng = np.random.default_rng(1)
    pts, nrm = surface_points(1 << 18, rng, noise=0.002)
    t0 = time.time()
    pool = rng.uniform(-1, 1, (1 << 21, 3)).astype(np.float32)
    pool_sdf = SignedDistance()(pool)
    print(f"signed-distance pool in {time.time() - t0:.0f} s", flush=True)
    dev = torch.device("cuda")
    surface = torch.from_numpy(np.concatenate([pts, nrm], 1).astype(np.float32)).to(dev)
    t1 = time.time()
    models, hist = train_three_levels(surface, torch.from_numpy(pool).to(dev),
                                      torch.from_numpy(pool_sdf).to(dev), steps=tuple(args.steps),
                                      batch=args.batch, deltas=(0.05, 0.01), precision="bf16",
                                      seed=1, check_every=50)
    torch.cuda.synchronize()
    for name, h in zip(("coarse", "medium", "fine"), hist):
        print(f"{name}: loss {h[0][1]:.4g} -> {min(v for _, v in h):.4g}", flush=True)
    out = {}
    for i, m in enumerate(models):
        for k, v in m.state_dict().items():
            out[f"L{i}.{k}"] = v.detach().cpu().numpy().astype(np.float32)
    out["omega"] = np.array([30.0, 30.0, 30.0], np.float32)
    np.savez(args.out, **out)
    print(f"trained in {time.time() - t1:.0f} s -> {args.out}")


if __name__ == "__main__":
    main()
