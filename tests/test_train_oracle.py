"""The training oracle against the reference's own autograd (golden loss
values and parameter gradients of loss_add_detail_fine) and against finite
differences of the loss in float64."""

import numpy as np
import torch

from conftest import golden, tiny_levels
from oracle import train as ot


def _fine():
    lf = golden("loss_fine.npz")
    params = [(lf[f"fine.net.{j}.0.weight"], lf[f"fine.net.{j}.0.bias"]) for j in range(4)]
    return lf, params, [30.0, 30.0, 30.0]


def test_oracle_loss_and_grads_match_reference_autograd():
    levels, _, _ = tiny_levels()
    lf, params, om = _fine()
    losses, grads = ot.residual_step_grads(params, om, levels[:2], lf["x"], lf["sdf"],
                                           lf["normals"])
    for k, v in losses.items():
        ref = float(lf["loss." + k])
        assert abs(v - ref) <= 1e-6 * abs(ref) + 1e-6, k
    for j in range(4):
        gw, gb = lf[f"grad.net.{j}.0.weight"], lf[f"grad.net.{j}.0.bias"]
        # the reference ran in float32: relative to the tensor's largest entry
        assert np.abs(grads[j][0] - gw).max() <= 2e-5 * np.abs(gw).max(), j
        assert np.abs(grads[j][1] - gb).max() <= 2e-5 * np.abs(gb).max(), j


def test_oracle_grads_match_finite_differences():
    levels, _, _ = tiny_levels()
    lf, params, om = _fine()
    args = (om, levels[:2], lf["x"], lf["sdf"], lf["normals"])
    _, grads = ot.residual_step_grads(params, *args)
    rng = np.random.default_rng(5)
    for trial in range(3):
        dirs = [(rng.standard_normal(np.shape(w)), rng.standard_normal(np.shape(b)))
                for w, b in params]
        h = 1e-6
        pp = [(w + h * dw, b + h * db) for (w, b), (dw, db) in zip(params, dirs)]
        pm = [(w - h * dw, b - h * db) for (w, b), (dw, db) in zip(params, dirs)]
        fd = (ot.residual_loss_total(pp, *args) - ot.residual_loss_total(pm, *args)) / (2 * h)
        an = sum((g[0] * dw).sum() + (g[1] * db).sum() for g, (dw, db) in zip(grads, dirs))
        assert abs(fd - an) <= 1e-5 * abs(an), (trial, fd, an)


def test_oracle_input_gradient_matches_finite_differences():
    lf, params, om = _fine()
    x = lf["x"][:8].astype(np.float64)
    _, g, _ = ot.forward_tangent(params, om, x)
    h = 1e-6
    for c in range(3):
        e = np.zeros(3)
        e[c] = h
        fp, _, _ = ot.forward_tangent(params, om, x + e)
        fm, _, _ = ot.forward_tangent(params, om, x - e)
        assert np.allclose((fp - fm) / (2 * h), g[:, c], rtol=1e-6, atol=1e-8)


def test_oracle_adam_matches_torch():
    rng = np.random.default_rng(2)
    p0 = rng.standard_normal(257)
    p = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([p], lr=1e-3, foreach=False)
    po, m, v = p0.copy(), np.zeros_like(p0), np.zeros_like(p0)
    for step in range(1, 5):
        g = rng.standard_normal(257)
        p.grad = torch.tensor(g)
        opt.step()
        po, m, v = ot.adam_update(po, g, m, v, step, lr=1e-3)
        assert np.allclose(p.detach().numpy(), po, rtol=0, atol=1e-12)


def test_oracle_training_batch_matches_reference():
    d = golden("train_batch.npz")
    for c in range(4):
        p, nr, s = ot.training_batch(d["vertices"], d[f"c{c}.idx"], d[f"c{c}.u"],
                                     float(d[f"c{c}.delta"]), bool(d[f"c{c}.neigh"]),
                                     bool(d[f"c{c}.dither"]))
        assert np.array_equal(p, d[f"c{c}.pts"]), c
        assert np.array_equal(nr, d[f"c{c}.normals"]), c
        assert np.array_equal(s, d[f"c{c}.sdf"]), c


def _true_sdf_case():
    d = golden("loss_true_sdf.npz")
    params = [(d[f"model.net.{j}.0.weight"], d[f"model.net.{j}.0.bias"]) for j in range(4)]
    return d, params, [30.0, 30.0, 30.0]


def test_oracle_true_sdf_matches_reference_autograd():
    d, params, om = _true_sdf_case()
    losses, grads = ot.true_sdf_step_grads(params, om, d["x"], d["sdf"], d["normals"])
    for k, v in losses.items():
        ref = float(d["loss." + k])
        assert abs(v - ref) <= 1e-5 * abs(ref), k
    for j in range(4):
        gw, gb = d[f"grad.net.{j}.0.weight"], d[f"grad.net.{j}.0.bias"]
        assert np.abs(grads[j][0] - gw).max() <= 2e-5 * np.abs(gw).max(), j
        assert np.abs(grads[j][1] - gb).max() <= 2e-5 * np.abs(gb).max(), j


def test_oracle_true_sdf_grads_match_finite_differences():
    d, params, om = _true_sdf_case()
    args = (om, d["x"], d["sdf"], d["normals"])
    _, grads = ot.true_sdf_step_grads(params, *args)
    rng = np.random.default_rng(9)
    dirs = [(rng.standard_normal(np.shape(w)), rng.standard_normal(np.shape(b)))
            for w, b in params]
    h = 1e-6
    pp = [(w + h * dw, b + h * db) for (w, b), (dw, db) in zip(params, dirs)]
    pm = [(w - h * dw, b - h * db) for (w, b), (dw, db) in zip(params, dirs)]
    fd = (ot.true_sdf_loss_total(pp, *args) - ot.true_sdf_loss_total(pm, *args)) / (2 * h)
    an = sum((g[0] * dw).sum() + (g[1] * db).sum() for g, (dw, db) in zip(grads, dirs))
    assert abs(fd - an) <= 1e-5 * abs(an)
