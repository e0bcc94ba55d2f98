"""FP64 evaluator of the SIREN levels, used only to state the error of results.

TEST INFRASTRUCTURE ONLY (see the package docstring).  Restates
i3d/model.py:107-129 in float64 with torch so it can run on the GPU for the
millions of points an error statement needs; it never produces a result the
library returns.
"""

from __future__ import annotations

import numpy as np
import torch


def level_params64(model, device):
    """(W, b) float64 pairs and omegas of an mplicits_gb300 / i3d SIREN."""
    lins = [blk[0] for blk in model.net]
    params = [(l.weight.detach().to(device, torch.float64),
               l.bias.detach().to(device, torch.float64)) for l in lins]
    omegas = [float(blk[1].w0) for blk in model.net[:-1]]
    return params, omegas


@torch.no_grad()
def forward64(params, omegas, x, chunk=1 << 19):
    """f(x) in float64 for x [P, 3] (any float dtype, any device)."""
    out = torch.empty(x.shape[0], dtype=torch.float64, device=x.device)
    for s in range(0, x.shape[0], chunk):
        h = x[s:s + chunk].to(torch.float64)
        for l, (W, b) in enumerate(params):
            h = torch.addmm(b, h, W.t())
            if l < len(params) - 1:
                h = torch.sin(omegas[l] * h)
        out[s:s + chunk] = h[:, 0]
    return out


def grid_xyz(N, index, device):
    """Reference grid coordinates (i3d/meshing.py:42-63) of int64 indices,
    computed with the same float32 operations as oracle.siren.grid_coords."""
    idx = index.to(torch.int64)
    fN = torch.tensor(float(N), dtype=torch.float32, device=device)
    idx_f = idx.to(torch.float32)
    s2 = (idx % N).to(torch.float32)
    q1 = idx_f / fN
    s1 = torch.fmod(q1, fN)
    s0 = torch.fmod(q1 / fN, fN)
    vs = torch.tensor(np.float32(2.0 / (N - 1)), device=device)
    return torch.stack([s0 * vs - 1.0, s1 * vs - 1.0, s2 * vs - 1.0], 1)


def chamfer_matched_upper(va, vb):
    """Upper bound of the pytorch3d Chamfer distance (mean squared nearest
    distance, summed over both directions) for two meshes with the same
    vertex count and canonical vertex order: each vertex's nearest neighbour
    is at most as far as its partner."""
    d2 = ((va.double() - vb.double()) ** 2).sum(1)
    return float(2.0 * d2.mean()) if d2.numel() else 0.0


def chamfer_kdtree(va, vb):
    """pytorch3d-style Chamfer distance through scipy k-d trees."""
    from scipy.spatial import cKDTree
    a = np.asarray(va, np.float64)
    b = np.asarray(vb, np.float64)
    if len(a) == 0 or len(b) == 0:
        return float("nan")
    da, _ = cKDTree(b).query(a, workers=-1)
    db, _ = cKDTree(a).query(b, workers=-1)
    return float((da ** 2).mean() + (db ** 2).mean())
