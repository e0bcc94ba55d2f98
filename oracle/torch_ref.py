"""Test infrastructure, not product code: the reference's training step as
the reference runs it, on the CPU with torch autograd, for the timed CPU
baseline of the training workload.

``PlainSiren`` has i3d.model.SIREN's layers (i3d/model.py:76-129: nn.Linear,
then sin(w0 x)); ``residual_loss`` restates ``loss_add_detail_fine``
(i3d/loss_functions.py:347-394) with the create_graph gradient of
i3d/diff_operators.py:259-265; ``train_step`` is the body of the fine
trainer's loop (experiment_scripts/train_sdf_on_neighborhood_fine.py:
235-252): zero_grad, forward, loss, backward, Adam.
"""

from __future__ import annotations

import torch
import torch.nn.functional as F


class PlainSiren(torch.nn.Module):
    def __init__(self, params, omegas):
        super().__init__()
        self.lins = torch.nn.ModuleList()
        for W, b in params:
            lin = torch.nn.Linear(W.shape[1], W.shape[0])
            with torch.no_grad():
                lin.weight.copy_(torch.as_tensor(W))
                lin.bias.copy_(torch.as_tensor(b))
            self.lins.append(lin)
        self.omegas = list(omegas)

    def forward(self, x):
        h = x
        for lin, w in zip(self.lins[:-1], self.omegas):
            h = torch.sin(w * lin(h))
        return self.lins[-1](h)


def _gradient(y, x):
    return torch.autograd.grad(y, [x], grad_outputs=torch.ones_like(y), create_graph=True)[0]


def residual_loss(fine, frozen, x, normals, sdf, weights=(3e3, 1e2, 5e1)):
    coords = x.clone().detach().requires_grad_(True)
    pred = fine(coords)
    g = _gradient(pred, coords)
    pg = g
    S = pred
    for m in frozen:
        c = x.clone().detach().requires_grad_(True)
        o = m(c)
        S = S + o
        pg = pg + _gradient(o, c).detach()
    sdf = sdf.reshape(-1, 1)
    sdf_c = torch.where(sdf != -1, (sdf - S) ** 2, torch.zeros_like(pred))
    nrm_c = torch.where(sdf != -1, 1 - F.cosine_similarity(normals, pg, dim=-1)[..., None],
                        torch.zeros_like(sdf))
    eik = ((pg.norm(dim=-1) - 1.0) ** 2).unsqueeze(-1)
    return sdf_c.mean() * weights[0] + nrm_c.mean() * weights[1] + eik.mean() * weights[2]


def train_step(fine, frozen, optim, x, normals, sdf):
    optim.zero_grad(set_to_none=True)
    loss = residual_loss(fine, frozen, x, normals, sdf)
    loss.backward()
    optim.step()
    return loss.detach()
