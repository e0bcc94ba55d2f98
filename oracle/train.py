"""Test infrastructure, not product code: the CPU oracle of the training step.

A float64 numpy restatement of the residual trainer's loss
(``loss_add_detail_fine``, i3d/loss_functions.py:347-394, with
``eikonal_constraint`` at i3d/loss_functions.py:41-42 and the gradient of
i3d/diff_operators.py:259-265) and of its parameter gradients, which the
reference obtains from autograd's double backward.  Here the input gradient
is carried in forward mode (a value row and three tangent rows per point,
i3d/model.py:107-129 differentiated by hand) and the weight gradients come
from one reverse pass over that graph.  Pinned by tests/golden/loss_fine.npz
(the reference's own loss values and ``p.grad`` after ``loss.backward()``) and
by central finite differences of the loss.  ``training_batch`` restates the
batch construction and is pinned bit for bit by tests/golden/train_batch.npz.

Adam follows torch.optim.Adam's single-tensor update (no weight decay).
"""

from __future__ import annotations

import numpy as np

DEFAULT_WEIGHTS = {"sdf_constraint": 3e3, "normal_constraint": 1e2, "grad_constraint": 5e1}
TRUE_SDF_WEIGHTS = {"sdf_on_surf": 3e3, "sdf_off_surf": 2e2, "normal_constraint": 1e2,
                    "grad_constraint": 5e1}


def forward_tangent(params, omegas, x):
    """f [n], df/dx [n, 3] and the per-layer pre-activations (value row with
    bias, tangent rows) of one level in float64."""
    x = np.asarray(x, np.float64)
    n = x.shape[0]
    v = x
    t = np.broadcast_to(np.eye(3), (n, 3, 3)).transpose(0, 2, 1)  # t[q, k, c] = dx_c/dx_k
    pres = []
    for (W, b), om in zip(params[:-1], omegas):
        W = np.asarray(W, np.float64)
        b = np.asarray(b, np.float64)
        av = v @ W.T + b
        at = t @ W.T  # [n, 3, out]
        pres.append((av, at))
        z = om * av
        v = np.sin(z)
        t = (om * np.cos(z))[:, None, :] * at
    WL = np.asarray(params[-1][0], np.float64)[0]
    bL = float(np.asarray(params[-1][1], np.float64)[0])
    f = v @ WL + bL
    g = t @ WL
    return f, g, pres


def residual_loss_seeds(f, g, F_frozen, G_frozen, gt_sdf, gt_normals, weights=None):
    """The three weighted loss terms and their derivatives with respect to
    this level's f and df/dx (the seeds of the reverse pass)."""
    w = dict(DEFAULT_WEIGHTS)
    if weights:
        w.update(weights)
    n = f.shape[0]
    S = f + F_frozen
    G = g + G_frozen
    gt_sdf = np.asarray(gt_sdf, np.float64).reshape(-1)
    N = np.asarray(gt_normals, np.float64)
    sup = gt_sdf != -1
    r = gt_sdf - S
    l_sdf = np.where(sup, r * r, 0.0)
    gl = np.linalg.norm(G, axis=1)
    nl = np.linalg.norm(N, axis=1)
    nn = np.maximum(nl, 1e-8)
    gg = np.maximum(gl, 1e-8)
    dot = np.sum(N * G, axis=1)
    cos = dot / (nn * gg)
    l_n = np.where(sup, 1.0 - cos, 0.0)
    l_e = (gl - 1.0) ** 2
    losses = {"sdf_constraint": w["sdf_constraint"] * l_sdf.mean(),
              "normal_constraint": w["normal_constraint"] * l_n.mean(),
              "grad_constraint": w["grad_constraint"] * l_e.mean()}
    phi = np.where(sup, -2.0 * r * w["sdf_constraint"] / n, 0.0)
    dcos = N / (nn * gg)[:, None] - np.where(gl > 1e-8, cos / (gg * gg), 0.0)[:, None] * G
    gam = np.where(sup[:, None], -w["normal_constraint"] / n * dcos, 0.0)
    safe = np.where(gl > 0, gl, 1.0)
    gam = gam + np.where((gl > 0)[:, None],
                         (2.0 * (gl - 1.0) * w["grad_constraint"] / n / safe)[:, None] * G, 0.0)
    return losses, phi, gam


def true_sdf_loss_seeds(f, g, gt_sdf, gt_normals, weights=None):
    """The coarse trainer's loss ``true_sdf`` (i3d/loss_functions.py:123-163,
    with sdf_constraint_on_surf, sdf_constraint_off_surf,
    vector_aligment_on_surf and eikonal_constraint at :9-42) and its seeds:
    pred^2 where gt == 0, (gt - pred)^2 elsewhere, 1 - cos(grad, n) where
    gt == 0, (|grad| - 1)^2 everywhere, each a mean over all points."""
    w = dict(TRUE_SDF_WEIGHTS)
    if weights:
        w.update(weights)
    n = f.shape[0]
    gt = np.asarray(gt_sdf, np.float64).reshape(-1)
    N = np.asarray(gt_normals, np.float64)
    on = gt == 0
    l_on = np.where(on, f * f, 0.0)
    r = gt - f
    l_off = np.where(on, 0.0, r * r)
    gl = np.linalg.norm(g, axis=1)
    nn = np.maximum(np.linalg.norm(N, axis=1), 1e-8)
    gg = np.maximum(gl, 1e-8)
    cos = np.sum(N * g, axis=1) / (nn * gg)
    l_n = np.where(on, 1.0 - cos, 0.0)
    l_e = (gl - 1.0) ** 2
    losses = {"sdf_on_surf": w["sdf_on_surf"] * l_on.mean(),
              "sdf_off_surf": w["sdf_off_surf"] * l_off.mean(),
              "normal_constraint": w["normal_constraint"] * l_n.mean(),
              "grad_constraint": w["grad_constraint"] * l_e.mean()}
    phi = np.where(on, 2.0 * f * w["sdf_on_surf"] / n, -2.0 * r * w["sdf_off_surf"] / n)
    dcos = N / (nn * gg)[:, None] - np.where(gl > 1e-8, cos / (gg * gg), 0.0)[:, None] * g
    gam = np.where(on[:, None], -w["normal_constraint"] / n * dcos, 0.0)
    safe = np.where(gl > 0, gl, 1.0)
    gam = gam + np.where((gl > 0)[:, None],
                         (2.0 * (gl - 1.0) * w["grad_constraint"] / n / safe)[:, None] * g, 0.0)
    return losses, phi, gam


def true_sdf_step_grads(params, omegas, x, gt_sdf, gt_normals, weights=None):
    f, g, _ = forward_tangent(params, omegas, x)
    losses, phi, gam = true_sdf_loss_seeds(f, g, gt_sdf, gt_normals, weights)
    return losses, param_grads(params, omegas, x, phi, gam)


def true_sdf_loss_total(params, omegas, x, gt_sdf, gt_normals, weights=None):
    f, g, _ = forward_tangent(params, omegas, x)
    return sum(true_sdf_loss_seeds(f, g, gt_sdf, gt_normals, weights)[0].values())


def param_grads(params, omegas, x, phi, gam):
    """Gradients of sum_q phi_q f_q + gam_q . g_q with respect to every
    (weight, bias), by reverse mode over the forward-mode graph."""
    x = np.asarray(x, np.float64)
    n = x.shape[0]
    _, _, pres = forward_tangent(params, omegas, x)
    L = len(params)
    grads = [None] * L
    # layer inputs: x for layer 0, (sin z, w cos z a_t) for the others
    ins = [(x, None)]
    for (av, at), om in zip(pres, omegas):
        z = om * av
        ins.append((np.sin(z), (om * np.cos(z))[:, None, :] * at))
    WL = np.asarray(params[-1][0], np.float64)[0]
    vL, tL = ins[-1]
    grads[-1] = ((phi @ vL + np.einsum("qk,qkj->j", gam, tL))[None, :], np.array([phi.sum()]))
    d_v = phi[:, None] * WL[None, :]
    d_t = gam[:, :, None] * WL[None, None, :]
    for l in range(L - 2, -1, -1):
        om = omegas[l]
        av, at = pres[l]
        z = om * av
        s, cz = np.sin(z), np.cos(z)
        da_t = (om * cz)[:, None, :] * d_t
        da_v = om * (d_v * cz - om * s * np.einsum("qkj,qkj->qj", d_t, at))
        vin, tin = ins[l]
        if l == 0:
            dW = da_v.T @ vin + da_t.sum(axis=0).T  # [out, 3]
        else:
            dW = da_v.T @ vin + np.einsum("qkj,qki->ji", da_t, tin)
        grads[l] = (dW, da_v.sum(axis=0))
        W = np.asarray(params[l][0], np.float64)
        d_v = da_v @ W
        d_t = da_t @ W
    return grads


def residual_step_grads(params, omegas, frozen, x, gt_sdf, gt_normals, weights=None):
    """Loss terms and parameter gradients of one residual training step.
    ``frozen`` is a list of (params, omegas) of the frozen levels."""
    f, g, _ = forward_tangent(params, omegas, x)
    F = np.zeros_like(f)
    G = np.zeros_like(g)
    for fp, fo in frozen:
        a, b, _ = forward_tangent(fp, fo, x)
        F += a
        G += b
    losses, phi, gam = residual_loss_seeds(f, g, F, G, gt_sdf, gt_normals, weights)
    return losses, param_grads(params, omegas, x, phi, gam)


def residual_loss_total(params, omegas, frozen, x, gt_sdf, gt_normals, weights=None):
    f, g, _ = forward_tangent(params, omegas, x)
    F = np.zeros_like(f)
    G = np.zeros_like(g)
    for fp, fo in frozen:
        a, b, _ = forward_tangent(fp, fo, x)
        F += a
        G += b
    losses, _, _ = residual_loss_seeds(f, g, F, G, gt_sdf, gt_normals, weights)
    return sum(losses.values())


def adam_update(p, g, m, v, step, lr=1e-4, beta1=0.9, beta2=0.999, eps=1e-8):
    """torch.optim.Adam's update of one tensor, in float64; returns (p, m, v)."""
    m = m + (1 - beta1) * (g - m)
    v = beta2 * v + (1 - beta2) * g * g
    bc1 = 1 - beta1 ** step
    bc2 = 1 - beta2 ** step
    denom = np.sqrt(v) / np.sqrt(bc2) + eps
    return p - (lr / bc1) * m / denom, m, v


def training_batch(vertices, idx, u, delta, use_neigh_delta=False, dithering=True,
                   delta_eps=0.0005):
    """create_training_data_on_neighborhood (experiment_scripts/utils.py:
    92-169) in float32 with the reference's operation order, given the
    sample indices ``idx`` (the randperm prefix, or all rows) and the
    uniforms ``u`` [n, 3] it draws.  Returns (pts, normals, sdf)."""
    f = np.float32
    surf = np.asarray(vertices, f)[np.asarray(idx)]
    n = surf.shape[0]
    u = np.asarray(u, f)
    if use_neigh_delta:
        dn = surf[:, -1:]
    else:
        dn = np.full((n, 1), f(delta_eps), f)
    xyz, nrm = surf[:, :3], surf[:, 3:6]
    off = xyz + (dn * u[:, 2:3]) * nrm
    pts = [xyz, off]
    normals = [nrm, nrm]
    sdf = [np.zeros(n, f), (dn[:, 0] * u[:, 2]).astype(f)]
    if dithering:
        pd = u * f(delta)
        pd = pd + (xyz + f(0.5 * delta) * nrm)
        pts.append(pd)
        normals.append(nrm)
        sdf.append(np.full(n, -1.0, f))
    return (np.concatenate(pts).astype(f), np.concatenate(normals).astype(f),
            np.concatenate(sdf).astype(f))
