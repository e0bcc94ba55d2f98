"""The hand-written training backward on the GPU against the reference's own
autograd (golden loss_add_detail_fine values and p.grad), the float64 oracle
(itself pinned by finite differences) and torch.optim.Adam."""

import ctypes

import numpy as np
import pytest
import torch
import torch.nn.functional as F

from conftest import golden, tiny_levels
from oracle import train as ot

pytestmark = pytest.mark.gpu


def _siren(sd, hidden, w0=30.0):
    from mplicits_gb300.model import SIREN
    m = SIREN(3, 1, hidden, w0=w0, delay_init=True)
    m.load_state_dict({k: torch.as_tensor(np.asarray(v)) for k, v in sd.items()})
    return m.cuda()


def _golden_setup():
    _, sds, _ = tiny_levels()
    lf = golden("loss_fine.npz")
    fine_sd = {k[5:]: lf[k] for k in lf.files if k.startswith("fine.")}
    fine = _siren(fine_sd, [32, 32, 32])
    frozen = [_siren(sds[0], [32, 32, 32]), _siren(sds[1], [32, 32, 32])]
    for m in frozen:
        m.eval()
        m.requires_grad_(False)
    x = torch.from_numpy(lf["x"]).cuda()
    nrm = torch.from_numpy(lf["normals"]).cuda()
    sdf = torch.from_numpy(lf["sdf"]).cuda()
    return lf, fine, frozen, x, nrm, sdf


def _check_grads(got, lf, rel):
    for j in range(4):
        gw, gb = lf[f"grad.net.{j}.0.weight"], lf[f"grad.net.{j}.0.bias"]
        w, b = got[2 * j].cpu().numpy(), got[2 * j + 1].cpu().numpy()
        assert w.shape == gw.shape and b.shape == gb.shape
        assert np.abs(w - gw).max() <= rel * np.abs(gw).max(), j
        assert np.abs(b - gb).max() <= rel * np.abs(gb).max(), j


def test_fused_trainer_loss_and_grads_match_reference_autograd(lib):
    from mplicits_gb300.train import ResidualTrainer
    lf, fine, frozen, x, nrm, sdf = _golden_setup()
    tr = ResidualTrainer(fine, frozen)
    losses, grads = tr.loss_and_grads(x, nrm, sdf)
    losses = losses.cpu().numpy()
    for i, k in enumerate(["sdf_constraint", "normal_constraint", "grad_constraint"]):
        ref = float(lf["loss." + k])
        assert abs(losses[i] - ref) <= 1e-4 * abs(ref), k
    _check_grads(grads, lf, 1e-4)


def _reference_loss(fine, frozen, x, nrm, sdf):
    """loss_add_detail_fine (i3d/loss_functions.py:347-394) written against
    the drop-in SIREN, with the gradient of i3d/diff_operators.py:259-265."""
    def gradient(y, xx):
        return torch.autograd.grad(y, [xx], grad_outputs=torch.ones_like(y),
                                   create_graph=True)[0]
    X = fine(x)
    coords, pred = X["model_in"], X["model_out"]
    g = gradient(pred, coords)
    terms = []
    for m in frozen:
        o = m(coords)
        terms.append((o["model_out"], gradient(o["model_out"], o["model_in"]).detach()))
    res_sdf, res_g = terms[1]
    co_sdf, co_g = terms[0]
    sdf_c = torch.where(sdf != -1, (sdf - pred - res_sdf - co_sdf) ** 2, torch.zeros_like(pred))
    pg = g + res_g + co_g
    nrm_c = torch.where(sdf != -1, 1 - F.cosine_similarity(nrm, pg, dim=-1)[..., None],
                        torch.zeros_like(sdf))
    eik = ((pg.norm(dim=-1) - 1.0) ** 2).unsqueeze(-1)
    return {"sdf_constraint": sdf_c.mean() * 3e3, "normal_constraint": nrm_c.mean() * 1e2,
            "grad_constraint": eik.mean() * 5e1}


def test_autograd_double_backward_matches_reference(lib):
    """The reference trainer's own code path: model(x), autograd.grad with
    create_graph=True, loss.backward() -- through the hand-written kernels."""
    lf, fine, frozen, x, nrm, sdf = _golden_setup()
    for m in frozen:
        m.requires_grad_(True)  # the reference leaves them trainable; grads unused
    losses = _reference_loss(fine, frozen, x, nrm, sdf)
    for k, v in losses.items():
        ref = float(lf["loss." + k])
        assert abs(float(v.detach()) - ref) <= 1e-4 * abs(ref), k
    sum(losses.values()).backward()
    _check_grads([p.grad for p in fine.parameters()], lf, 1e-4)


def test_input_gradient_hessian_term_matches_autograd_free_oracle(lib):
    """d/dx of sum dg . df/dx (the coordinate leaf's gradient under the
    double backward) against float64 finite differences of the oracle."""
    from mplicits_gb300.train import param_grads
    lf, fine, _, x, _, _ = _golden_setup()
    dg = torch.randn(x.shape[0], 3, device="cuda", generator=torch.Generator("cuda").manual_seed(1))
    _, dx = param_grads(fine, x, dg=dg, want_dx=True)
    params = [(lf[f"fine.net.{j}.0.weight"], lf[f"fine.net.{j}.0.bias"]) for j in range(4)]
    xs = lf["x"].astype(np.float64)
    dgn = dg.cpu().numpy().astype(np.float64)
    h = 1e-6
    ref = np.zeros_like(xs)
    for c in range(3):
        e = np.zeros(3)
        e[c] = h
        _, gp, _ = ot.forward_tangent(params, [30.0] * 3, xs + e)
        _, gm, _ = ot.forward_tangent(params, [30.0] * 3, xs - e)
        ref[:, c] = np.sum(dgn * (gp - gm) / (2 * h), axis=1)
    got = dx.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()


def _random_level(widths, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    params = []
    dims = [3] + widths + [1]
    for i in range(len(dims) - 1):
        fan = dims[i]
        lim = (1.0 / fan) if i == 0 else (np.sqrt(6.0 / fan) / 30.0)
        W = rng.uniform(-lim, lim, (dims[i + 1], fan)).astype(np.float32) * (scale if i else 1)
        b = rng.uniform(-0.05, 0.05, dims[i + 1]).astype(np.float32)
        params.append((W, b))
    sd = {}
    for j, (W, b) in enumerate(params):
        sd[f"net.{j}.0.weight"] = W
        sd[f"net.{j}.0.bias"] = b
    return params, sd


@pytest.mark.parametrize("width,n", [(256, 3000), (128, 4099), (64, 777)])
def test_wide_level_grads_match_oracle(lib, width, n):
    """Full-width levels, ragged point counts: kernel gradients against the
    float64 oracle (relative to each tensor's largest entry)."""
    from mplicits_gb300.train import ResidualTrainer
    params, sd = _random_level([width] * 3, 10 + width, scale=2.0)
    fparams, fsd = _random_level([128] * 3, 3, scale=2.0)
    fine = _siren(sd, [width] * 3)
    frozen = [_siren(fsd, [128] * 3).eval()]
    rng = np.random.default_rng(n)
    xs = rng.uniform(-0.9, 0.9, (n, 3)).astype(np.float32)
    nrm = xs / np.linalg.norm(xs, axis=1, keepdims=True)
    sdf = rng.uniform(-0.02, 0.02, (n, 1)).astype(np.float32)
    sdf[rng.random(n) < 0.4] = -1.0
    tr = ResidualTrainer(fine, frozen)
    losses, grads = tr.loss_and_grads(torch.from_numpy(xs).cuda(), torch.from_numpy(nrm).cuda(),
                                      torch.from_numpy(sdf).cuda())
    ref_l, ref_g = ot.residual_step_grads(params, [30.0] * 3, [(fparams, [30.0] * 3)], xs, sdf,
                                          nrm)
    lo = losses.cpu().numpy()
    for i, k in enumerate(["sdf_constraint", "normal_constraint", "grad_constraint"]):
        assert abs(lo[i] - ref_l[k]) <= 1e-4 * abs(ref_l[k]) + 1e-6, k
    for j in range(4):
        for t in range(2):
            got = grads[2 * j + t].cpu().numpy().astype(np.float64)
            ref = ref_g[j][t].reshape(got.shape)
            assert np.abs(got - ref).max() <= 2e-4 * np.abs(ref).max(), (j, t)


def test_adam_kernel_matches_torch_adam(lib):
    from mplicits_gb300 import capi
    g = torch.Generator("cuda").manual_seed(4)
    shapes = [(256, 3), (256,), (256, 256), (1, 256), (1,)]
    ps = [torch.randn(s, device="cuda", generator=g) for s in shapes]
    ref = [p.clone().requires_grad_(True) for p in ps]
    opt = torch.optim.Adam(ref, lr=1e-4)
    ms = [torch.zeros_like(p) for p in ps]
    vs = [torch.zeros_like(p) for p in ps]
    P = ctypes.c_void_p
    for step in range(1, 6):
        grads = [torch.randn(s, device="cuda", generator=g) for s in shapes]
        for r, gr in zip(ref, grads):
            r.grad = gr.clone()
        opt.step()
        cnt = len(ps)
        capi.check(lib.mpl_adam_step(
            cnt, (P * cnt)(*[p.data_ptr() for p in ps]), (P * cnt)(*[x.data_ptr() for x in grads]),
            (P * cnt)(*[m.data_ptr() for m in ms]), (P * cnt)(*[v.data_ptr() for v in vs]),
            (ctypes.c_int64 * cnt)(*[p.numel() for p in ps]), 1e-4, 0.9, 0.999, 1e-8, step,
            capi.stream_ptr()), "mpl_adam_step")
        for p, r in zip(ps, ref):
            assert torch.allclose(p, r.detach(), rtol=0, atol=2e-7), step


def test_trainer_steps_follow_oracle(lib):
    """Three Adam steps of the fused trainer against three float64 oracle
    steps from the same start."""
    from mplicits_gb300.train import ResidualTrainer
    lf, fine, frozen, x, nrm, sdf = _golden_setup()
    levels, _, _ = tiny_levels()
    params = [(lf[f"fine.net.{j}.0.weight"].astype(np.float64),
               lf[f"fine.net.{j}.0.bias"].astype(np.float64)) for j in range(4)]
    ms = [(np.zeros_like(w), np.zeros_like(b)) for w, b in params]
    vs = [(np.zeros_like(w), np.zeros_like(b)) for w, b in params]
    tr = ResidualTrainer(fine, frozen, lr=1e-4)
    for step in range(1, 4):
        tr.step(x, nrm, sdf)
        _, grads = ot.residual_step_grads(params, [30.0] * 3, levels[:2], lf["x"], lf["sdf"],
                                          lf["normals"])
        new = []
        for j in range(4):
            w, mw, vw = ot.adam_update(params[j][0], grads[j][0], ms[j][0], vs[j][0], step)
            b, mb, vb = ot.adam_update(params[j][1], grads[j][1], ms[j][1], vs[j][1], step)
            new.append((w, b))
            ms[j], vs[j] = (mw, mb), (vw, vb)
        params = new
    got = [p.detach().cpu().numpy() for p in fine.parameters()]
    for j in range(4):
        for t in range(2):
            start = lf[f"fine.net.{j}.0.{'weight' if t == 0 else 'bias'}"]
            moved = np.abs(params[j][t] - start).max()
            assert moved > 0
            # Adam moves each entry by about lr * sign(m); entries whose
            # gradient is near zero may take the other sign in float32
            off = np.abs(got[2 * j + t] - params[j][t]) > 0.02 * moved
            assert off.mean() <= 0.01, (j, t, off.mean())


def test_batch_kernel_matches_reference_bit_exact(lib):
    """mpl_train_batch given the reference's own draws reproduces
    create_training_data_on_neighborhood's batch bit for bit."""
    from mplicits_gb300 import capi
    d = golden("train_batch.npz")
    V = torch.from_numpy(d["vertices"]).cuda()
    for c in range(4):
        idx = torch.from_numpy(d[f"c{c}.idx"]).cuda()
        u = torch.from_numpy(d[f"c{c}.u"]).cuda()
        n = idx.shape[0]
        dither = bool(d[f"c{c}.dither"])
        rows = 3 * n if dither else 2 * n
        pts = torch.empty(rows, 3, device="cuda")
        nrm = torch.empty(rows, 3, device="cuda")
        sdf = torch.empty(rows, device="cuda")
        flags = (capi.MPL_BATCH_NEIGH_DELTA if bool(d[f"c{c}.neigh"]) else 0) | \
            (capi.MPL_BATCH_DITHER if dither else 0)
        capi.check(lib.mpl_train_batch(capi.ptr(V), V.shape[0], V.shape[1], capi.ptr(idx),
                                       capi.ptr(u), n, float(d[f"c{c}.delta"]), 0.0005, flags, 0,
                                       capi.ptr(pts), capi.ptr(nrm), capi.ptr(sdf),
                                       capi.stream_ptr()), "mpl_train_batch")
        assert np.array_equal(pts.cpu().numpy(), d[f"c{c}.pts"]), c
        assert np.array_equal(nrm.cpu().numpy(), d[f"c{c}.normals"]), c
        assert np.array_equal(sdf.cpu().numpy(), d[f"c{c}.sdf"]), c
    assert capi.device_status() == capi.MPL_OK


def test_batch_drop_in_uses_torch_draws(lib):
    from mplicits_gb300.train import create_training_data_on_neighborhood
    d = golden("train_batch.npz")
    V = torch.from_numpy(d["vertices"]).cuda()
    torch.manual_seed(77)
    out = create_training_data_on_neighborhood(V, 50, device="cuda", delta=0.01,
                                               use_neigh_delta=True)
    torch.manual_seed(77)
    idx = torch.randperm(V.shape[0], device="cuda")[:50].cpu().numpy()
    u = torch.rand((50, 3)).numpy()
    ref = ot.training_batch(d["vertices"], idx, u, 0.01, True, True)
    for got, want in zip(out["on_surf"], ref):
        assert np.array_equal(got.cpu().numpy(), want)


def test_batch_device_generator(lib):
    from mplicits_gb300.train import create_training_data_on_neighborhood
    d = golden("train_batch.npz")
    V = torch.from_numpy(d["vertices"]).cuda()
    a = create_training_data_on_neighborhood(V, 200, delta=0.01, seed=5)["on_surf"]
    b = create_training_data_on_neighborhood(V, 200, delta=0.01, seed=5)["on_surf"]
    c = create_training_data_on_neighborhood(V, 200, delta=0.01, seed=6)["on_surf"]
    assert all(torch.equal(x, y) for x, y in zip(a, b))
    assert not torch.equal(a[0], c[0])
    pts, nrm, sdf = [t.cpu().numpy() for t in a]
    vset = {tuple(r) for r in d["vertices"][:, :3].tolist()}
    assert all(tuple(r) in vset for r in pts[:200].tolist())
    assert np.all(sdf[:200] == 0) and np.all(sdf[400:] == -1)
    assert np.all((sdf[200:400] >= 0) & (sdf[200:400] < 0.0005))
    # offset rows lie on the normal line at the recorded distance
    off = pts[200:400] - pts[:200]
    assert np.allclose(off, sdf[200:400, None] * nrm[:200], atol=1e-7)
    dith = pts[400:] - pts[:200] - 0.005 * nrm[:200]
    assert np.all((dith >= -1e-6) & (dith < 0.01 + 1e-6))


def test_true_sdf_trainer_matches_reference_autograd(lib):
    """The coarse trainer's loss (true_sdf) on the plain kernels against the
    reference's own loss values and p.grad (golden loss_true_sdf.npz)."""
    from mplicits_gb300.train import ResidualTrainer
    d = golden("loss_true_sdf.npz")
    sd = {k[6:]: d[k] for k in d.files if k.startswith("model.")}
    model = _siren(sd, [32, 32, 32])
    tr = ResidualTrainer(model, loss="true_sdf")
    losses, grads = tr.loss_and_grads(torch.from_numpy(d["x"]).cuda(),
                                      torch.from_numpy(d["normals"]).cuda(),
                                      torch.from_numpy(d["sdf"]).cuda())
    losses = losses.cpu().numpy()
    assert tr.names == ["sdf_on_surf", "sdf_off_surf", "normal_constraint", "grad_constraint"]
    for i, k in enumerate(tr.names):
        ref = float(d["loss." + k])
        assert abs(losses[i] - ref) <= 1e-4 * abs(ref), k
    for j in range(4):
        gw, gb = d[f"grad.net.{j}.0.weight"], d[f"grad.net.{j}.0.bias"]
        assert np.abs(grads[2 * j].cpu().numpy() - gw).max() <= 1e-4 * np.abs(gw).max(), j
        assert np.abs(grads[2 * j + 1].cpu().numpy() - gb).max() <= 1e-4 * np.abs(gb).max(), j
