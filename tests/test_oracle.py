"""The oracle against the golden vectors made from the reference's own code
(tests/golden/make_golden.py), and the marching-cubes oracle's invariants."""

import hashlib

import numpy as np
import pytest
import torch

from conftest import golden, tiny_levels
from oracle import mc, siren


@pytest.mark.parametrize("N", [2, 3, 4, 5, 16, 127, 128])
def test_grid_matches_reference(N):
    g = golden("grid.npz")
    c = siren.grid_coords(N, 2.0 / (N - 1))
    assert hashlib.sha256(c.tobytes()).hexdigest() == str(g[f"sha_{N}"])
    assert np.array_equal(c[g[f"idx_{N}"]], g[f"xyz_{N}"])


def test_grid_512_sampled_rows_match_reference():
    # the full 512^3 hash is checked on the GPU grid; here the sampled rows
    g = golden("grid.npz")
    idx = g["idx_512"]
    assert np.array_equal(siren.grid_coords(512, 2.0 / 511, idx), g["xyz_512"])


def test_band_compare_is_float32():
    b = golden("band_compare.npz")
    assert np.array_equal(siren.band_mask(b["S"], float(b["delta"])), b["mask"])


def _cfg1_params():
    from mplicits_gb300.model import SIREN
    torch.manual_seed(0)
    m = SIREN(3, 1, [256, 256, 256], w0=30)
    sd = {k: v.numpy() for k, v in m.state_dict().items()}
    return m, sd


def test_package_init_reproduces_reference_weights():
    g = golden("siren_cfg1_probe.npz")
    _, sd = _cfg1_params()
    for k, v in sd.items():
        assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == str(g[f"sha_{k}"]), k


def test_siren_forward_matches_reference_fp32_and_fp64():
    g = golden("siren_cfg1_probe.npz")
    _, sd = _cfg1_params()
    params = siren.params_from_state_dict(sd)
    om = [30.0, 30.0, 30.0]
    for x, y in ((g["x16"], g["y16"]), (g["xr"], g["yr"])):
        y32 = siren.siren_forward(params, om, x)
        y64 = siren.siren_forward(params, om, x, np.float64)
        assert np.abs(y32 - y).max() < 1e-5
        assert np.abs(y64 - y).max() < 1e-5


def test_input_grad_matches_reference_autograd():
    g = golden("siren_cfg1_probe.npz")
    _, sd = _cfg1_params()
    params = siren.params_from_state_dict(sd)
    gr = siren.siren_input_grad(params, [30.0] * 3, g["xr"][:256])
    ref = g["grad_r"]
    assert np.abs(gr - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())


def test_multistage_matches_reference_loop():
    levels, _, d = tiny_levels()
    N = int(d["N"])
    deltas = [float(x) for x in d["deltas"]]
    S, bands = siren.multistage_sdf(levels, deltas, N, chunk=32 ** 3 // 8)
    assert np.abs(S - d["S_banded"]).max() <= 1e-6
    grid = siren.grid_coords(N, 2.0 / (N - 1))
    for i, b in enumerate(bands, start=1):
        got = {tuple(r) for r in grid[b].tolist()}
        ref = {tuple(r) for r in d[f"band{i}_pts"].tolist()}
        assert got == ref
    S_full, _ = siren.multistage_sdf(levels, [], N)
    assert np.abs(S_full - d["S_full"]).max() <= 1e-6


def _sphere(N, r=0.6):
    x = np.linspace(-1, 1, N, dtype=np.float32)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    return (np.sqrt(X ** 2 + Y ** 2 + Z ** 2) - r).astype(np.float32)


def _edge_use(faces):
    use = {}
    for tri in faces:
        for a, b in ((tri[0], tri[1]), (tri[1], tri[2]), (tri[2], tri[0])):
            use[(a, b)] = use.get((a, b), 0) + 1
    return use


@pytest.mark.parametrize("N", [8, 33])
def test_oracle_mc_closed_oriented_sphere(N):
    v, f, n, val = mc.marching_cubes_raw(_sphere(N), 0.0, 2.0 / (N - 1), (-1, -1, -1))
    use = _edge_use(f)
    assert all(c == 1 and use.get((b, a)) == 1 for (a, b), c in use.items())
    assert v.shape[0] - len(use) // 2 + f.shape[0] == 2  # Euler characteristic
    c = v[f].mean(1)
    nrm = np.cross(v[f][:, 1] - v[f][:, 0], v[f][:, 2] - v[f][:, 0])
    assert ((nrm * c).sum(1) > 0).all()
    assert ((n * v).sum(1) > 0).all()


def test_oracle_mc_random_field_is_manifold():
    rng = np.random.default_rng(3)
    S = rng.standard_normal((12, 12, 12)).astype(np.float32)
    S[0], S[-1], S[:, 0], S[:, -1], S[:, :, 0], S[:, :, -1] = 1, 1, 1, 1, 1, 1
    v, f, _, _ = mc.marching_cubes_raw(S)
    use = _edge_use(f)
    assert all(c == 1 and use.get((b, a)) == 1 for (a, b), c in use.items())


def test_oracle_mc_empty_when_level_out_of_range(capsys):
    v, f, n, val = mc.marching_cubes(np.ones((4, 4, 4), np.float32), [-1, -1, -1], 0.5)
    assert v.shape[0] == 0 and f.shape[0] == 0
    assert "Surface level must be within volume data range." in capsys.readouterr().out


def test_mc_header_matches_generator():
    from mplicits_gb300 import mc_tables
    with open(mc_tables.HEADER_PATH) as fh:
        assert fh.read() == mc_tables.render_header()


def test_mc_table_complementary_cases_mirror():
    from mplicits_gb300.mc_tables import build_tables
    count, table = build_tables()
    # without ambiguous faces a case and its complement cut the same edges
    for case in range(256):
        e1 = set(table[case][table[case] >= 0].tolist())
        e2 = set(table[255 - case][table[255 - case] >= 0].tolist())
        assert e1 == e2
