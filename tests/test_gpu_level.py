"""Fused level kernel (FP32 plain form) and band compaction through the C ABI,
against the reference's golden outputs and the numpy oracle."""

import ctypes
import hashlib

import numpy as np
import pytest
import torch

from conftest import golden, tiny_levels
from oracle import siren

pytestmark = pytest.mark.gpu

TOL = 1e-5  # plain form vs the reference PyTorch FP32 path (absolute)


def _model(sd, width_cfg, w0=30.0, precision="fp32"):
    from mplicits_gb300.model import SIREN
    m = SIREN(3, 1, width_cfg, w0=w0, delay_init=True, precision=precision)
    m.load_state_dict({k: torch.as_tensor(np.asarray(v)) for k, v in sd.items()})
    return m.cuda().eval()


def _cfg1():
    from mplicits_gb300.model import SIREN
    torch.manual_seed(0)
    m = SIREN(3, 1, [256, 256, 256], w0=30)
    sd = {k: v.numpy().copy() for k, v in m.state_dict().items()}
    return m.cuda().eval(), siren.params_from_state_dict(sd)


def test_cfg1_level_matches_reference_outputs(lib):
    from mplicits_gb300.model import level_forward
    g = golden("siren_cfg1_probe.npz")
    m, _ = _cfg1()
    for x, y in ((g["x16"], g["y16"]), (g["xr"], g["yr"])):
        out = level_forward(m, torch.from_numpy(x).cuda()).cpu().numpy()
        assert np.abs(out - y).max() <= TOL


def test_forward_dict_contract(lib):
    m, params = _cfg1()
    x = torch.rand(1000, 3, device="cuda") * 2 - 1
    with torch.no_grad():
        out = m(x)
    assert set(out) == {"model_in", "model_out"}
    assert out["model_out"].shape == (1000, 1)
    assert out["model_in"].requires_grad and out["model_in"] is not x
    ref = siren.siren_forward(params, [30.0] * 3, x.cpu().numpy())
    assert np.abs(out["model_out"][:, 0].cpu().numpy() - ref).max() <= TOL


@pytest.mark.parametrize("cfg", [[256, 256, 256], [128, 128], [32, 32, 32], [100, 60, 17],
                                 [64], [256, 256, 256, 256, 256]])
@pytest.mark.parametrize("P", [1, 127, 128, 129, 5000])
def test_widths_and_ragged_sizes(lib, cfg, P):
    from mplicits_gb300.model import SIREN, level_forward
    torch.manual_seed(len(cfg) * 1000 + sum(cfg))
    m = SIREN(3, 1, cfg, w0=30).cuda().eval()
    params = siren.params_from_state_dict({k: v.cpu().numpy() for k, v in m.state_dict().items()})
    rng = np.random.default_rng(P)
    x = rng.uniform(-1, 1, (P, 3)).astype(np.float32)
    out = level_forward(m, torch.from_numpy(x).cuda()).cpu().numpy()
    ref = siren.siren_forward(params, m.omegas(), x, np.float64)
    assert np.abs(out - ref).max() <= TOL


def test_empty_point_set_is_a_no_op(lib):
    from mplicits_gb300.model import level_forward
    m, _ = _cfg1()
    S = torch.full((4,), 7.0, device="cuda")
    level_forward(m, torch.zeros(0, 3, device="cuda"), S=S[:0])
    torch.cuda.synchronize()
    assert (S == 7.0).all()


def _run_level(lib, m, points, n, S, mode, index=None, n_dev=None, band=None):
    from mplicits_gb300 import capi
    net, packed = m.packed()
    capi.check(lib.mpl_level_forward(ctypes.byref(net), capi.ptr(packed), ctypes.byref(points),
                                     capi.ptr(index), capi.ptr(n_dev), n, capi.ptr(S), mode,
                                     None if band is None else ctypes.byref(band),
                                     capi.MPL_FP32, capi.stream_ptr()), "level")


def test_grid_points_are_the_reference_grid(lib):
    from mplicits_gb300 import capi
    from mplicits_gb300.meshing import _grid_points
    g = golden("grid.npz")
    for N in (2, 3, 4, 5, 16, 127, 128, 512):
        pts = _grid_points(N, 2.0 / (N - 1))
        n = N ** 3
        out = torch.empty(n, 3, device="cuda")
        capi.check(lib.mpl_grid_points(ctypes.byref(pts), None, n, capi.ptr(out),
                                       capi.stream_ptr()), "grid")
        h = hashlib.sha256(out.cpu().numpy().tobytes()).hexdigest()
        assert h == str(g[f"sha_{N}"]), N


@pytest.mark.parametrize("N", [1000, 1290, 1291, 1300])
def test_grid_points_of_large_grids_match_the_oracle(lib, N):
    """Indexed grid points of grids too large to write whole, up to the
    largest N the exact 32-bit path covers (1290) and past it (the 64-bit
    path), against the oracle's float32 restatement of i3d/meshing.py:42-63."""
    from mplicits_gb300 import capi
    from mplicits_gb300.meshing import _grid_points
    rng = np.random.default_rng(N)
    idx = np.concatenate([rng.integers(0, N ** 3, 200000), [0, N ** 3 - 1, N * N - 1, N * N,
                                                             N ** 3 - N]])
    idx = idx[idx < 2 ** 31].astype(np.int32)
    pts = _grid_points(N, 2.0 / (N - 1))
    out = torch.empty(idx.shape[0], 3, device="cuda")
    ti = torch.from_numpy(idx).cuda()
    capi.check(lib.mpl_grid_points(ctypes.byref(pts), capi.ptr(ti), idx.shape[0], capi.ptr(out),
                                   capi.stream_ptr()), "grid")
    ref = siren.grid_coords(N, 2.0 / (N - 1), idx.astype(np.int64))
    assert np.array_equal(out.cpu().numpy().view(np.uint32), ref.view(np.uint32))


def test_grid_mode_index_accumulate_and_fused_band(lib):
    """Grid points generated in-kernel, an index list, a device count,
    accumulation and the fused band list, all against the oracle."""
    from mplicits_gb300 import capi
    from mplicits_gb300.meshing import _grid_points
    levels, sds, d = tiny_levels()
    N = 24
    n = N ** 3
    m0 = _model(sds[0], [32, 32, 32])
    m1 = _model(sds[1], [32, 32, 32])
    pts = _grid_points(N, 2.0 / (N - 1))
    S = torch.empty(n, device="cuda")
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    band = capi.MplBand(delta=0.05, out_index=out.data_ptr(), count_dev=cnt.data_ptr(), capacity=n)
    _run_level(lib, m0, pts, n, S, capi.MPL_STORE, band=band)
    S0 = S.cpu().numpy().copy()
    grid = siren.grid_coords(N, 2.0 / (N - 1))
    ref0 = siren.siren_forward(*levels[0], grid, np.float64)
    assert np.abs(S0 - ref0).max() <= TOL
    k = int(cnt.item())
    got = np.sort(out[:k].cpu().numpy())
    assert np.array_equal(got, np.nonzero(np.abs(S0) < np.float32(0.05))[0])
    # level 1 on the band list, count read on the device
    out2 = torch.empty(n, dtype=torch.int32, device="cuda")
    cnt2 = torch.zeros(1, dtype=torch.int32, device="cuda")
    band2 = capi.MplBand(delta=0.02, out_index=out2.data_ptr(), count_dev=cnt2.data_ptr(),
                         capacity=n)
    _run_level(lib, m1, pts, n, S, capi.MPL_ACCUMULATE, index=out, n_dev=cnt, band=band2)
    S1 = S.cpu().numpy()
    idx = np.nonzero(np.abs(S0) < np.float32(0.05))[0]
    ref1 = S0.astype(np.float64).copy()
    ref1[idx] += siren.siren_forward(*levels[1], grid[idx], np.float64)
    assert np.abs(S1 - ref1).max() <= TOL
    untouched = np.setdiff1d(np.arange(n), idx)
    assert np.array_equal(S1[untouched], S0[untouched])
    k2 = int(cnt2.item())
    got2 = np.sort(out2[:k2].cpu().numpy())
    exp2 = idx[np.abs(S1[idx]) < np.float32(0.02)]
    assert np.array_equal(got2, exp2)
    from mplicits_gb300 import capi as c
    assert c.device_status() == c.MPL_OK


def test_band_capacity_overflow_is_counted(lib):
    from mplicits_gb300 import capi
    S = torch.zeros(1000, device="cuda")
    out = torch.full((10,), -1, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    band = capi.MplBand(delta=1.0, out_index=out.data_ptr(), count_dev=cnt.data_ptr(), capacity=10)
    capi.check(lib.mpl_band_compact(capi.ptr(S), None, None, 1000, ctypes.byref(band),
                                    capi.stream_ptr()), "band")
    assert int(cnt.item()) == 1000  # > capacity: overflow reported
    assert (out.cpu() >= 0).all()


def test_band_compact_matches_reference_mask(lib):
    """Standalone compaction on the reference's own comparison vector and
    on random values with an index list and a device-side count."""
    from mplicits_gb300 import capi
    b = golden("band_compare.npz")
    S = torch.from_numpy(b["S"]).cuda()
    n = S.numel()
    out = torch.empty(n, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    band = capi.MplBand(delta=float(b["delta"]), out_index=out.data_ptr(),
                        count_dev=cnt.data_ptr(), capacity=n)
    capi.check(lib.mpl_band_compact(capi.ptr(S), None, None, n, ctypes.byref(band),
                                    capi.stream_ptr()), "band")
    k = int(cnt.item())
    mask = np.zeros(n, bool)
    mask[out[:k].cpu().numpy()] = True
    assert np.array_equal(mask, b["mask"])
    rng = np.random.default_rng(5)
    Sr = rng.uniform(-0.2, 0.2, 1 << 20).astype(np.float32)
    idx = np.sort(rng.choice(Sr.size, 300000, replace=False)).astype(np.int32)
    St = torch.from_numpy(Sr).cuda()
    it = torch.from_numpy(idx).cuda()
    ndev = torch.tensor([200000], dtype=torch.int32, device="cuda")
    out = torch.empty(300000, dtype=torch.int32, device="cuda")
    band = capi.MplBand(delta=0.05, out_index=out.data_ptr(), count_dev=cnt.data_ptr(),
                        capacity=300000)
    capi.check(lib.mpl_band_compact(capi.ptr(St), capi.ptr(it), capi.ptr(ndev), 300000,
                                    ctypes.byref(band), capi.stream_ptr()), "band")
    k = int(cnt.item())
    got = np.sort(out[:k].cpu().numpy())
    sel = idx[:200000]
    assert np.array_equal(got, sel[np.abs(Sr[sel]) < np.float32(0.05)])


def test_cpu_tensors_raise():
    from mplicits_gb300.model import SIREN
    m = SIREN(3, 1, [32, 32], w0=30)
    with pytest.raises(RuntimeError):
        with torch.no_grad():
            m(torch.zeros(4, 3))
