"""BF16 tcgen05 level kernel: exactness of the tensor-core arithmetic
(against a numpy emulation of the same BF16 roundings) and its error
against the FP64 oracle."""

import numpy as np
import pytest
import torch

from oracle import siren

pytestmark = pytest.mark.gpu


def bf16_round(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def f16_round(a):
    return np.asarray(a, np.float32).astype(np.float16).astype(np.float64)


def emulate_bf16_level(params, omegas, x, rnd=bf16_round):
    """The kernel's arithmetic in float64: FP32-phase layer 0 with omega
    folded, 16-bit activations and 16-bit omega*W in the hidden GEMMs (``rnd``
    rounds to BF16 or FP16), FP32 sines into the output layer."""
    W0, b0 = params[0]
    z = np.asarray(x, np.float64) @ (omegas[0] * W0.astype(np.float64)).T + omegas[0] * b0
    s = np.sin(z)
    for l in range(1, len(params) - 1):
        W, b = params[l]
        Wq = rnd(np.float32(omegas[l]) * W.astype(np.float32))
        z = rnd(s.astype(np.float32)) @ Wq.T + omegas[l] * b.astype(np.float64)
        s = np.sin(z)
    Wl, bl = params[-1]
    return (s @ Wl.astype(np.float64).T + bl)[:, 0]


def _model(cfg, seed):
    from mplicits_gb300.model import SIREN
    torch.manual_seed(seed)
    m = SIREN(3, 1, cfg, w0=30, precision="bf16").cuda().eval()
    params = siren.params_from_state_dict({k: v.cpu().numpy() for k, v in m.state_dict().items()})
    return m, params


@pytest.fixture(params=[16, 32], ids=["unit16", "unit32"])
def epilogue_unit(request, lib):
    from mplicits_gb300 import capi
    old = capi.get_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT)
    capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, request.param)
    yield request.param
    capi.set_option(capi.MPL_OPT_BF16_EPILOGUE_UNIT, old)


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
@pytest.mark.parametrize("cfg", [[256, 256, 256], [128, 128, 128], [64, 64], [100, 60, 17],
                                 [256, 256, 256, 256, 256]])
@pytest.mark.parametrize("P", [1, 200, 20000])
def test_bf16_tensor_core_arithmetic_is_exact(lib, epilogue_unit, cfg, P, prec):
    from mplicits_gb300.model import level_forward
    m, params = _model(cfg, 7 + len(cfg))
    rng = np.random.default_rng(P)
    x = rng.uniform(-1, 1, (P, 3)).astype(np.float32)
    out = level_forward(m, torch.from_numpy(x).cuda(), precision=prec).cpu().numpy()
    emu = emulate_bf16_level(params, m.omegas(), x, bf16_round if prec == "bf16" else f16_round)
    # exact up to accumulation order and the hardware sine (~1e-6 for these
    # phases); a BF16 rounding flip of an activation moves a rare point by up
    # to ~1e-3.  A wrong descriptor or tile layout gives O(1) errors.
    err = np.abs(out - emu)
    if P >= 100:
        assert np.median(err) <= 5e-6
    assert err.max() <= 1e-3
    from mplicits_gb300 import capi
    assert capi.device_status() == capi.MPL_OK


def test_bf16_error_against_fp64_oracle_cfg1(lib):
    from mplicits_gb300.model import level_forward
    m, params = _model([256, 256, 256], 0)
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (1 << 16, 3)).astype(np.float32)
    out = level_forward(m, torch.from_numpy(x).cuda(), precision="bf16").cpu().numpy()
    ref = siren.siren_forward(params, m.omegas(), x, np.float64)
    err = np.abs(out - ref)
    print(f"bf16 vs fp64: max {err.max():.3e} rms {np.sqrt((err ** 2).mean()):.3e}")
    assert err.max() <= 5e-3


def test_bf16_grid_band_pipeline_matches_fp32_bands_where_clear(lib):
    """Grid mode + fused band in BF16: every point whose BF16 value is
    farther than the error margin from delta gets the FP32 decision."""
    from mplicits_gb300.meshing import BandedReconstruction
    m, params = _model([256, 256, 256], 3)
    rec32 = BandedReconstruction([m, m], [0.05], 48, "cuda", precision="fp32")
    rec16 = BandedReconstruction([m, m], [0.05], 48, "cuda", precision="bf16")
    rec32.sample()
    rec16.sample()
    S0 = BandedReconstruction([m], [], 48, "cuda", precision="fp32").sample().cpu().numpy()
    k32 = rec32.band_sizes()[0]
    k16 = rec16.band_sizes()[0]
    b32 = set(rec32.band_index[0][:k32].cpu().tolist())
    b16 = set(rec16.band_index[0][:k16].cpu().tolist())
    diff = b32 ^ b16
    assert all(abs(abs(S0[p]) - 0.05) < 5e-3 for p in diff)


def test_fp16_operands_meet_the_error_target_on_trained_levels(lib):
    """The trained three-level fixture: FP16 operands keep every level within
    5e-4 of the FP64 oracle (BF16 does not in the far field)."""
    from mplicits_gb300.model import SIREN, level_forward
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "three_level_sphere.npz"))
    x = np.random.default_rng(4).uniform(-1, 1, (1 << 17, 3)).astype(np.float32)
    for i in range(3):
        sd = {k[3:]: d[k] for k in d.files if k.startswith(f"L{i}.")}
        m = SIREN(3, 1, [256, 256, 256], w0=30, delay_init=True, precision="fp16")
        m.load_state_dict({k: torch.from_numpy(v) for k, v in sd.items()})
        m = m.cuda().eval()
        params = siren.params_from_state_dict({k: v.cpu().numpy() for k, v in m.state_dict().items()})
        out = level_forward(m, torch.from_numpy(x).cuda()).cpu().numpy()
        ref = siren.siren_forward(params, m.omegas(), x, np.float64)
        assert np.abs(out - ref).max() <= 5e-4, i


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
@pytest.mark.parametrize("cfg", [[256, 256, 256], [128, 128, 128], [64, 64], [100, 60, 17],
                                 [256, 256, 256, 256, 256]])
@pytest.mark.parametrize("P", [1, 129, 777, 40000])
def test_two_tile_kernel_equals_single_tile_kernel(lib, epilogue_unit, cfg, P, prec):
    """The two-tiles-per-CTA kernel computes every element with the single-
    tile kernel's arithmetic: values, gradients and band lists are identical."""
    from mplicits_gb300 import capi
    from mplicits_gb300.grad import level_gradient
    from mplicits_gb300.model import level_forward
    m, _ = _model(cfg, 11 + len(cfg))
    rng = np.random.default_rng(P + 1)
    x = torch.from_numpy(rng.uniform(-1, 1, (P, 3)).astype(np.float32)).cuda()
    out = {}
    # single tile; two tiles with the first layer in the drains; two tiles
    # with first-layer warps.  Gradients in forward mode (the tangent rows of
    # these kernels) and in reverse mode.
    for tiles, l0w in ((1, 0), (2, 0), (2, 4), (2, 8)):
        capi.set_option(capi.MPL_OPT_TC_TILES_IN_FLIGHT, tiles)
        capi.set_option(capi.MPL_OPT_TC_LAYER0_WARPS, l0w)
        try:
            S = level_forward(m, x, precision=prec).clone()
            Sg, G = level_gradient(m, x, precision=prec)
            capi.set_option(capi.MPL_OPT_TC_GRAD_REVERSE, 0)
            Sf, Gf = level_gradient(m, x, precision=prec)
            out[(tiles, l0w)] = (S, Sg.clone(), G.clone(), Sf.clone(), Gf.clone())
        finally:
            capi.set_option(capi.MPL_OPT_TC_TILES_IN_FLIGHT, 2)
            capi.set_option(capi.MPL_OPT_TC_LAYER0_WARPS, 8)
            capi.set_option(capi.MPL_OPT_TC_GRAD_REVERSE, 1)
    for k in ((2, 0), (2, 4), (2, 8)):
        for a, b in zip(out[(1, 0)], out[k]):
            assert torch.equal(a, b), k
    assert capi.device_status() == capi.MPL_OK


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
@pytest.mark.parametrize("N", [40, 97, 128])
def test_layer0_warps_grid_bands_and_point_lists(lib, epilogue_unit, prec, N):
    """The first-layer-warp kernel against the kernel that computes the
    first layer in its drains, on the paths the reconstruction takes: grid
    points with a fused band list, then index lists whose count lives on the
    device, accumulating into S.  Values and band lists are identical."""
    from mplicits_gb300 import capi
    from mplicits_gb300.meshing import BandedReconstruction
    levels = [_model([256, 256, 256], 31 + i)[0] for i in range(3)]
    for lv, sc in zip(levels[1:], (0.1, 0.02)):
        with torch.no_grad():
            lv.net[-1][0].weight.mul_(sc)
    res = {}
    for l0w in (0, 4, 8):
        capi.set_option(capi.MPL_OPT_TC_LAYER0_WARPS, l0w)
        try:
            rec = BandedReconstruction(levels, [0.3, 0.1], N, "cuda", prec)
            rec.sample()
            sizes = rec.band_sizes()
            bands = [torch.sort(rec.band_index[i][:sizes[i]])[0] for i in range(2)]
            res[l0w] = (rec.S.clone(), bands, sizes)
        finally:
            capi.set_option(capi.MPL_OPT_TC_LAYER0_WARPS, 8)
    for k in (4, 8):
        assert res[0][2] == res[k][2] and min(res[0][2]) > 0
        assert torch.equal(res[0][0], res[k][0])
        for a, b in zip(res[0][1], res[k][1]):
            assert torch.equal(a, b)
    assert capi.device_status() == capi.MPL_OK
