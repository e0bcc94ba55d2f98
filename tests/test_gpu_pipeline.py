"""The three-stage training on the GPU kernels: each stage lowers its loss
and the trained nested model fits the synthetic surface."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_three_stage_training_fits_the_surface(lib):
    from mplicits_gb300.pipeline import train_three_levels
    from mplicits_gb300.synthetic import SignedDistance, surface_points
    rng = np.random.default_rng(1)
    pts, nrm = surface_points(1 << 15, rng, noise=0.0)
    surface = torch.from_numpy(np.concatenate([pts, nrm], 1)).cuda()
    pool = rng.uniform(-1, 1, (1 << 14, 3)).astype(np.float32)
    sdf = SignedDistance(n_dense=1 << 17)(pool)
    models, hist = train_three_levels(surface, torch.from_numpy(pool).cuda(),
                                      torch.from_numpy(sdf).cuda(), steps=(300, 150, 150),
                                      batch=4096, width=128, check_every=25)
    for h in hist:
        assert h[-1][1] < h[0][1], h
    # the nested sum vanishes on the surface far better than the coarse level alone
    x = torch.from_numpy(surface_points(4096, np.random.default_rng(7))[0]).cuda()
    from mplicits_gb300.model import level_forward
    S0 = level_forward(models[0], x, precision="fp32")
    S = S0.clone()
    for m in models[1:]:
        level_forward(m, x, S=S, accumulate=True, precision="fp32")
    torch.cuda.synchronize()
    e0, e = S0.abs().mean().item(), S.abs().mean().item()
    print("mean |S| on the surface: coarse", e0, "nested", e)
    assert e0 < 0.01 and e < e0


def test_three_stage_training_with_neighbourhood_deltas(lib):
    """The reference scripts' band sizing: delta = 1.3 max |f_frozen(v)| and
    per-vertex calc_deltas radii on the mesh's scene."""
    from mplicits_gb300.pipeline import frozen_max_dist, train_three_levels
    from mplicits_gb300.scene import RaycastingScene, calc_deltas
    from mplicits_gb300.synthetic import SignedDistance, surface_mesh
    pos, nrm, faces = surface_mesh(64, 128)
    surface = torch.from_numpy(np.concatenate([pos, nrm], 1)).cuda()
    scene = RaycastingScene(pos, faces)
    rng = np.random.default_rng(2)
    pool = rng.uniform(-1, 1, (1 << 14, 3)).astype(np.float32)
    sdf = SignedDistance(n_dense=1 << 17)(pool)
    models, hist = train_three_levels(surface, torch.from_numpy(pool).cuda(),
                                      torch.from_numpy(sdf).cuda(), steps=(300, 100, 100),
                                      batch=4096, width=128, check_every=25,
                                      deltas=(None, None), scene=scene, neighborhood_delta=True)
    for h in hist:
        assert h[-1][1] < h[0][1], h
    # the radii the medium stage trained on: calc_deltas with max_delta = max_dist
    md = frozen_max_dist(models[:1], surface)
    out = calc_deltas(surface, scene, max_delta=md, n_iters=100)
    d = out[:, 6]
    assert out.shape == (surface.shape[0], 7)
    assert float(d.min()) > 0 and float(d.max()) <= float(md) * 1.02 + 1e-6
