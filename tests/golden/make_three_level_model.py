"""Train the three-level residual model of the 512^3 band-culled workload.

    python tests/golden/make_three_level_model.py [--steps 4000 2000 2000] [--device cuda]

Each level is 3 -> 256 x 3 -> 1 with omega0 = 30, trained with torch autograd
on the synthetic surface of ``mplicits_gb300.synthetic`` (2^18 surface points,
Gaussian noise sigma = 0.002, seed 1) with the reference trainers' step
semantics:

  coarse  train_sdf.py:238-269 with the ``true_sdf`` loss
          (i3d/loss_functions.py:123-163): surface points (sdf 0, normals)
          plus uniform off-surface points with their signed distance;
  medium  train_sdf_on_neighborhood*.py with ``loss_add_detail``
          (i3d/loss_functions.py:263-323), coarse level frozen;
  fine    with ``loss_add_detail_fine`` (i3d/loss_functions.py:327-394),
          coarse and medium frozen.
Residual batches follow create_training_data_on_neighborhood
(experiment_scripts/utils.py:92-169): n surface points (sdf 0), n points
offset along the normal by delta_eps * u (sdf delta_eps * u), n dithered
points flagged sdf = -1.  Adam, lr 1e-4; the best-loss state after 10 %
warm-up is kept.  Output: three_level_sphere.npz (omega not baked).
"""

from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np
import torch
import torch.nn.functional as F

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mplicits_gb300.synthetic import SignedDistance, surface_points  # noqa: E402


class Siren(torch.nn.Module):
    """Plain torch SIREN with the i3d.model.SIREN parameter layout."""

    def __init__(self, width=256, depth=3, w0=30.0):
        super().__init__()
        from mplicits_gb300.model import SIREN
        self.m = SIREN(3, 1, [width] * depth, w0=w0)
        self.w0 = w0

    def forward(self, x):
        h = x
        for blk in self.m.net[:-1]:
            h = torch.sin(self.w0 * blk[0](h))
        return self.m.net[-1][0](h)


def grad(y, x):
    return torch.autograd.grad(y, [x], grad_outputs=torch.ones_like(y), create_graph=True)[0]


def train_coarse(steps, pts, nrm, pool_x, pool_sdf, batch, gen, dev):
    """pts/nrm: surface samples, pool_x/pool_sdf: uniform off-surface samples
    with their signed distance, all resident on ``dev``."""
    model = Siren().to(dev)
    opt = torch.optim.Adam(model.parameters(), lr=1e-4)
    best, best_state = float("inf"), None
    zeros = torch.zeros(batch, 1, device=dev)
    for step in range(steps):
        i = torch.randint(0, pts.shape[0], (batch,), device=dev, generator=gen)
        j = torch.randint(0, pool_x.shape[0], (batch,), device=dev, generator=gen)
        x = torch.cat([pts[i], pool_x[j]]).requires_grad_(True)
        gt_sdf = torch.cat([zeros, pool_sdf[j][:, None]])
        gt_n = torch.cat([nrm[i], torch.zeros(batch, 3, device=dev)])
        y = model(x)
        g = grad(y, x)
        on = gt_sdf == 0
        loss = (torch.where(on, y ** 2, torch.zeros_like(y)).mean() * 3e3 +
                torch.where(~on, (gt_sdf - y) ** 2, torch.zeros_like(y)).mean() * 2e2 +
                torch.where(on, 1 - F.cosine_similarity(g, gt_n, dim=-1)[:, None],
                            torch.zeros_like(y)).mean() * 1e2 +
                ((g.norm(dim=-1) - 1) ** 2).mean() * 5e1)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        lv = loss.item()
        if step > steps // 10 and lv < best:
            best, best_state = lv, {k: v.detach().clone() for k, v in model.state_dict().items()}
        if step % 500 == 0:
            print(f"coarse {step} {lv:.4f}", flush=True)
    model.load_state_dict(best_state)
    return model


def residual_batch(pts, nrm, n, delta, gen, delta_eps=0.0005):
    dev = pts.device
    i = torch.randint(0, pts.shape[0], (n,), device=dev, generator=gen)
    s, nr = pts[i], nrm[i]
    u = torch.rand(n, 3, device=dev, generator=gen)
    off = s + delta_eps * u[:, -1:] * nr
    dith = u * delta + s + 0.5 * delta * nr
    x = torch.cat([s, off, dith])
    normals = torch.cat([nr, nr, nr])
    sdf = torch.cat([torch.zeros(n, device=dev), delta_eps * u[:, -1],
                     -torch.ones(n, device=dev)])
    return x, normals, sdf


def train_residual(steps, frozen, pts, nrm, delta, batch, gen, dev):
    model = Siren().to(dev)
    opt = torch.optim.Adam(model.parameters(), lr=1e-4)
    best, best_state = float("inf"), None
    for step in range(steps):
        xb, gt_n, sb = residual_batch(pts, nrm, batch, delta, gen)
        x = xb.requires_grad_(True)
        gt_sdf = sb[:, None]
        y = model(x)
        g = grad(y, x)
        fsum, gsum = 0.0, 0.0
        for fm in frozen:
            xf = x.detach().clone().requires_grad_(True)
            yf = fm(xf)
            gf = grad(yf, xf).detach()
            fsum = fsum + yf.detach()
            gsum = gsum + gf
        sup = gt_sdf != -1
        pg = g + gsum
        loss = (torch.where(sup, (gt_sdf - y - fsum) ** 2, torch.zeros_like(y)).mean() * 3e3 +
                torch.where(sup, 1 - F.cosine_similarity(gt_n, pg, dim=-1)[:, None],
                            torch.zeros_like(y)).mean() * 1e2 +
                ((pg.norm(dim=-1) - 1) ** 2).mean() * 5e1)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        lv = loss.item()
        if step > steps // 10 and lv < best:
            best, best_state = lv, {k: v.detach().clone() for k, v in model.state_dict().items()}
        if step % 500 == 0:
            print(f"residual {step} {lv:.4f}", flush=True)
    model.load_state_dict(best_state)
    return model


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, nargs=3, default=[4000, 2000, 2000])
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--device", default="cuda" if torch.cuda.is_available() else "cpu")
    ap.add_argument("--out", default=os.path.join(HERE, "three_level_sphere.npz"))
    args = ap.parse_args()
    torch.set_num_threads(max(1, os.cpu_count() or 1))
    torch.manual_seed(1)
    rng = np.random.default_rng(1)
    pts_np, nrm_np = surface_points(1 << 18, rng, noise=0.002)
    t0 = time.time()
    # off-surface pool: uniform points and their signed distance, computed once
    pool_np = rng.uniform(-1, 1, (1 << 21, 3)).astype(np.float32)
    pool_sdf_np = SignedDistance()(pool_np)
    print(f"signed-distance pool in {time.time() - t0:.0f} s", flush=True)
    dev = torch.device(args.device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(1)
    pts = torch.from_numpy(pts_np).to(dev)
    nrm = torch.from_numpy(nrm_np).to(dev)
    pool_x = torch.from_numpy(pool_np).to(dev)
    pool_sdf = torch.from_numpy(pool_sdf_np).to(dev)
    coarse = train_coarse(args.steps[0], pts, nrm, pool_x, pool_sdf, args.batch, gen, dev)
    print(f"coarse done at {time.time() - t0:.0f} s", flush=True)
    medium = train_residual(args.steps[1], [coarse], pts, nrm, 0.05, args.batch // 2, gen, dev)
    fine = train_residual(args.steps[2], [coarse, medium], pts, nrm, 0.01, args.batch // 2, gen,
                          dev)
    out = {}
    for i, lv in enumerate((coarse, medium, fine)):
        for k, v in lv.m.state_dict().items():
            out[f"L{i}.{k}"] = v.cpu().numpy().astype(np.float32)
    out["omega"] = np.array([30.0, 30.0, 30.0], np.float32)
    np.savez(args.out, **out)
    print(f"trained in {time.time() - t0:.0f} s -> {args.out}")


if __name__ == "__main__":
    main()
