"""Reverse-mode input gradient on the tensor cores: f and df/dx from a
backward sweep over each tile of 128 points, against the FP64 oracle and the
forward-mode tangent rows of the level kernels (same values, different
16-bit roundings), with point lists, accumulation and fused band lists."""

import numpy as np
import pytest
import torch

from oracle import siren

pytestmark = pytest.mark.gpu


def _model(cfg, seed, precision):
    from mplicits_gb300.model import SIREN
    torch.manual_seed(seed)
    m = SIREN(3, 1, cfg, w0=30, precision=precision).cuda().eval()
    params = siren.params_from_state_dict({k: v.cpu().numpy() for k, v in m.state_dict().items()})
    return m, params


def _grads(m, x, reverse, **kw):
    from mplicits_gb300 import capi
    from mplicits_gb300.grad import level_gradient
    capi.set_option(capi.MPL_OPT_TC_GRAD_REVERSE, 1 if reverse else 0)
    try:
        S, G = level_gradient(m, x, **kw)
        torch.cuda.synchronize()
        return S.clone(), G.clone()
    finally:
        capi.set_option(capi.MPL_OPT_TC_GRAD_REVERSE, 1)


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
@pytest.mark.parametrize("cfg", [[256, 256, 256], [128, 128, 128], [64, 64], [100, 60, 17]])
@pytest.mark.parametrize("P", [1, 127, 129, 20000])
def test_reverse_gradient_vs_fp64_and_forward_mode(lib, prec, cfg, P):
    from mplicits_gb300 import capi
    m, params = _model(cfg, 5, prec)
    x = np.random.default_rng(P).uniform(-1, 1, (P, 3)).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    S_r, G_r = _grads(m, xt, True)
    S_f, G_f = _grads(m, xt, False)
    assert capi.device_status() == capi.MPL_OK
    ref = siren.siren_input_grad(params, m.omegas(), x)
    f64 = siren.siren_forward(params, m.omegas(), x, np.float64)
    norm = np.maximum(np.linalg.norm(ref, axis=1), 1e-3)
    e_r = np.linalg.norm(G_r.cpu().numpy() - ref, axis=1) / norm
    e_f = np.linalg.norm(G_f.cpu().numpy() - ref, axis=1) / norm
    tol = 2e-2 if prec == "bf16" else 4e-3
    print(f"{prec} {cfg} P={P}: median relative error reverse {np.median(e_r):.2e}, "
          f"forward {np.median(e_f):.2e}")
    assert np.median(e_r) <= tol
    if P >= 1000:  # the 16-bit roundings sit on adjoints instead of tangents
        assert np.median(e_r) <= 3.0 * np.median(e_f)
    # the value is the forward pass of the level kernels: identical
    assert torch.equal(S_r, S_f)
    assert np.abs(S_r.cpu().numpy() - f64).max() <= 5e-3


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_reverse_gradient_index_accumulate_and_band(lib, prec):
    from mplicits_gb300 import capi
    from mplicits_gb300.grad import level_gradient
    m0, p0 = _model([256, 256, 256], 1, prec)
    m1, p1 = _model([256, 256, 256], 2, prec)
    x = np.random.default_rng(3).uniform(-1, 1, (5000, 3)).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    S, G = level_gradient(m0, xt)
    idx = torch.arange(0, 5000, 3, dtype=torch.int32, device="cuda")
    level_gradient(m1, xt, S=S, G=G, accumulate=True, index=idx, n=idx.numel())
    torch.cuda.synchronize()
    assert capi.device_status() == capi.MPL_OK
    ref = siren.siren_input_grad(p0, m0.omegas(), x)
    sel = np.arange(0, 5000, 3)
    ref[sel] += siren.siren_input_grad(p1, m1.omegas(), x[sel])
    norm = np.maximum(np.linalg.norm(ref, axis=1), 1e-3)
    err = np.linalg.norm(G.cpu().numpy() - ref, axis=1) / norm
    assert np.median(err) <= (2e-2 if prec == "bf16" else 4e-3)
    # S and its band list are the forward kernel's, reverse mode or not
    S2, _ = _grads(m0, xt, False)
    S1, _ = _grads(m0, xt, True)
    assert torch.equal(S1, S2)
