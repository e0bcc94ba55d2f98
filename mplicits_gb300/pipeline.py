"""The three-stage training of a nested model on the GPU kernels.

The reference trains the coarse level with ``true_sdf`` (train_sdf.py:
219-268: surface points with SDF 0 and normals, domain points with their
signed distance), then the medium level against the frozen coarse one with
``loss_add_detail`` (experiment_scripts/train_sdf_on_neighborhood.py), then
the fine level against both with ``loss_add_detail_fine``
(experiment_scripts/train_sdf_on_neighborhood_fine.py:220-262), each with
Adam at lr 1e-4 and the best-loss state after a warm-up kept.  Here every
step runs on ``ResidualTrainer`` (hand-written forward, loss, double
backward and Adam) and the residual batches on the batch kernel; only the
best-loss check reads the loss back, every ``check_every`` steps.

The residual stages can size their band as the reference scripts do
(experiment_scripts/train_sdf_on_neighborhood.py:165-185 and
train_sdf_on_neighborhood_fine.py:159-183): max_dist = max |f_frozen(v)|
over the vertices, batch delta = 1.3 max_dist, and, with the neighbourhood
option, per-vertex deltas from ``calc_deltas`` on the mesh's scene with
max_delta = max_dist (medium) or 1.3 max_dist (fine).
"""

from __future__ import annotations

import torch

from .model import SIREN, level_forward
from .scene import calc_deltas
from .train import ResidualTrainer, create_training_data_on_neighborhood


def _new_level(width, depth, w0, precision, device, seed):
    torch.manual_seed(seed)
    return SIREN(3, 1, [width] * depth, w0=w0, precision=precision).to(device)


def _run(trainer, batch_fn, steps, check_every, warmup_frac, log):
    best, best_state, history = float("inf"), None, []
    warm = int(steps * warmup_frac)
    for step in range(steps):
        losses = trainer.step(*batch_fn(step))
        if (step + 1) % check_every == 0 or step == steps - 1:
            total = float(losses.sum())
            history.append((step, total))
            if log:
                log(step, total)
            if step >= warm and total < best:
                best = total
                best_state = {k: v.detach().clone() for k, v in trainer.model.state_dict().items()}
    if best_state is not None:
        trainer.model.load_state_dict(best_state)
    return history


def train_coarse(surface, pool_x, pool_sdf, steps, batch, width=256, depth=3, w0=30,
                 precision="bf16", seed=0, check_every=50, warmup_frac=0.1, log=None):
    """Coarse level with true_sdf.  ``surface`` [M, 6] (xyz, normal),
    ``pool_x`` [P, 3] / ``pool_sdf`` [P] domain points with their signed
    distance, all on the training device.  Each step: ``batch`` surface and
    ``batch`` domain points."""
    dev = surface.device
    model = _new_level(width, depth, w0, precision, dev, seed)
    tr = ResidualTrainer(model, lr=1e-4, precision=precision, loss="true_sdf")
    gen = torch.Generator(dev).manual_seed(seed + 1)
    zeros3 = torch.zeros(batch, 3, device=dev)
    zeros1 = torch.zeros(batch, device=dev)

    def batch_fn(step):
        i = torch.randint(0, surface.shape[0], (batch,), device=dev, generator=gen)
        j = torch.randint(0, pool_x.shape[0], (batch,), device=dev, generator=gen)
        x = torch.cat([surface[i, :3], pool_x[j]])
        n = torch.cat([surface[i, 3:6], zeros3])
        s = torch.cat([zeros1, pool_sdf[j]])
        return x, n, s

    history = _run(tr, batch_fn, steps, check_every, warmup_frac, log)
    return model, history


def frozen_max_dist(frozen, vertices):
    """max |sum of the frozen levels| over the vertices [M, >= 3] (a 0-d
    float32 tensor on their device), as the reference scripts compute it
    with the frozen models under no_grad."""
    x = vertices[:, :3].contiguous()
    S = None
    for i, m in enumerate(frozen):
        S = level_forward(m, x, S, accumulate=i > 0)
    return S.abs().max()


def train_residual(surface, frozen, steps, batch, delta, width=256, depth=3, w0=30,
                   precision="bf16", seed=0, check_every=50, warmup_frac=0.1, log=None,
                   scene=None, neighborhood_delta=False, fine=False):
    """A residual level against the frozen ``frozen`` levels, on batches of
    create_training_data_on_neighborhood with neighbourhood ``delta``.

    ``delta=None`` takes 1.3 max |f_frozen(v)| over the surface rows.  With
    ``neighborhood_delta`` the surface rows must be the vertices of the mesh
    in ``scene`` (a ``scene.RaycastingScene``); each gets its calc_deltas
    radius (max_delta = max_dist, or 1.3 max_dist when ``fine``) and the
    batches use it.  Returns (model, loss history)."""
    dev = surface.device
    max_dist = None
    if delta is None or neighborhood_delta:
        max_dist = frozen_max_dist(frozen, surface)
    if delta is None:
        delta = float(max_dist * 1.3)
    if neighborhood_delta:
        if scene is None:
            raise ValueError("neighborhood_delta needs the mesh's scene")
        surface = calc_deltas(surface[:, :6], scene, max_delta=max_dist * 1.3 if fine else max_dist,
                              n_iters=100)
    model = _new_level(width, depth, w0, precision, dev, seed)
    tr = ResidualTrainer(model, list(frozen), lr=1e-4, precision=precision)

    def batch_fn(step):
        return create_training_data_on_neighborhood(surface, batch, device=dev, delta=delta,
                                                    use_neigh_delta=neighborhood_delta,
                                                    seed=seed * 1000003 + step)["on_surf"]

    history = _run(tr, batch_fn, steps, check_every, warmup_frac, log)
    return model, history


def train_three_levels(surface, pool_x, pool_sdf, steps=(4000, 2000, 2000), batch=1 << 16,
                       deltas=(0.05, 0.01), width=256, depth=3, w0=30, precision="bf16", seed=0,
                       check_every=50, log=None, scene=None, neighborhood_delta=False):
    """Coarse (true_sdf), medium (residual, delta0) and fine (residual,
    delta1) levels; returns the three models and their loss histories.
    ``deltas=(None, None)`` sizes the bands from the frozen levels' error as
    the reference scripts do; ``scene`` + ``neighborhood_delta`` add the
    per-vertex calc_deltas radii (``surface`` then holds the mesh's vertices
    and normals)."""
    coarse, h0 = train_coarse(surface, pool_x, pool_sdf, steps[0], batch, width, depth, w0,
                              precision, seed, check_every, log=log)
    coarse.eval()
    medium, h1 = train_residual(surface, [coarse], steps[1], batch, deltas[0], width, depth, w0,
                                precision, seed + 1, check_every, log=log, scene=scene,
                                neighborhood_delta=neighborhood_delta)
    medium.eval()
    fine, h2 = train_residual(surface, [coarse, medium], steps[2], batch, deltas[1], width, depth,
                              w0, precision, seed + 2, check_every, log=log, scene=scene,
                              neighborhood_delta=neighborhood_delta, fine=True)
    fine.eval()
    return [coarse, medium, fine], [h0, h1, h2]
