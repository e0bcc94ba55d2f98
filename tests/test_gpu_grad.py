"""Input gradients (normals) from the fused forward-mode kernels, against the
reference's autograd golden vectors and the FP64 oracle."""

import numpy as np
import pytest
import torch

from conftest import golden
from oracle import siren

pytestmark = pytest.mark.gpu


def _model(cfg, seed, precision="fp32"):
    from mplicits_gb300.model import SIREN
    torch.manual_seed(seed)
    m = SIREN(3, 1, cfg, w0=30, precision=precision).cuda().eval()
    params = siren.params_from_state_dict({k: v.cpu().numpy() for k, v in m.state_dict().items()})
    return m, params


def test_fp32_gradient_matches_reference_autograd(lib):
    from mplicits_gb300.grad import level_gradient
    g = golden("siren_cfg1_probe.npz")
    m, _ = _model([256, 256, 256], 0)
    S, G = level_gradient(m, torch.from_numpy(g["xr"][:256]).cuda())
    ref = g["grad_r"]
    assert np.abs(G.cpu().numpy() - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())
    assert np.abs(S.cpu().numpy() - g["yr"][:256]).max() <= 1e-5


@pytest.mark.parametrize("cfg", [[256, 256, 256], [128, 128], [100, 60, 17], [64]])
@pytest.mark.parametrize("P", [1, 31, 33, 4000])
def test_fp32_gradient_vs_fp64(lib, cfg, P):
    from mplicits_gb300.grad import level_gradient
    m, params = _model(cfg, P + len(cfg))
    x = np.random.default_rng(P).uniform(-1, 1, (P, 3)).astype(np.float32)
    S, G = level_gradient(m, torch.from_numpy(x).cuda())
    ref = siren.siren_input_grad(params, m.omegas(), x)
    scale = max(1.0, np.abs(ref).max())
    assert np.abs(G.cpu().numpy() - ref).max() <= 2e-5 * scale
    assert np.abs(S.cpu().numpy() - siren.siren_forward(params, m.omegas(), x, np.float64)).max() <= 1e-5


@pytest.mark.parametrize("unit", [16, 32])
@pytest.mark.parametrize("cfg", [[256, 256, 256], [128, 128, 128], [64, 64]])
def test_bf16_gradient_vs_fp64(lib, cfg, unit):
    from mplicits_gb300 import capi
    old = capi.get_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT)
    capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, unit)
    from mplicits_gb300.grad import level_gradient
    m, params = _model(cfg, 5, precision="bf16")
    x = np.random.default_rng(9).uniform(-1, 1, (20000, 3)).astype(np.float32)
    S, G = level_gradient(m, torch.from_numpy(x).cuda())
    ref = siren.siren_input_grad(params, m.omegas(), x)
    err = np.linalg.norm(G.cpu().numpy() - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-3)
    print(f"bf16 gradient relative error: median {np.median(err):.2e} max {err.max():.2e}")
    assert np.median(err) <= 2e-2
    f64 = siren.siren_forward(params, m.omegas(), x, np.float64)
    assert np.abs(S.cpu().numpy() - f64).max() <= 5e-3
    assert capi.device_status() == capi.MPL_OK
    capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, old)


def test_autograd_input_gradient_through_forward(lib):
    """torch.autograd.grad(model_out, model_in) on the drop-in module."""
    g = golden("siren_cfg1_probe.npz")
    m, _ = _model([256, 256, 256], 0)
    for p in m.parameters():
        p.requires_grad_(False)
    out = m(torch.from_numpy(g["xr"][:256]).cuda())
    gx = torch.autograd.grad(out["model_out"], [out["model_in"]],
                             grad_outputs=torch.ones_like(out["model_out"]))[0]
    ref = g["grad_r"]
    assert np.abs(gx.cpu().numpy() - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())


def test_gradient_accumulates_over_levels_with_index(lib):
    from mplicits_gb300.grad import level_gradient
    m0, p0 = _model([64, 64], 1)
    m1, p1 = _model([64, 64], 2)
    x = np.random.default_rng(3).uniform(-1, 1, (1000, 3)).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    S, G = level_gradient(m0, xt)
    idx = torch.arange(0, 1000, 3, dtype=torch.int32, device="cuda")
    level_gradient(m1, xt, S=S, G=G, accumulate=True, index=idx, n=idx.numel())
    ref = siren.siren_input_grad(p0, m0.omegas(), x)
    sel = np.arange(0, 1000, 3)
    ref[sel] += siren.siren_input_grad(p1, m1.omegas(), x[sel])
    assert np.abs(G.cpu().numpy() - ref).max() <= 2e-5 * max(1.0, np.abs(ref).max())
