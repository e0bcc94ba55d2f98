"""The band-culled pipeline (drop-in create_mesh_multistage) against the
reference loop's own output volume and band lists."""

import os

import numpy as np
import pytest
import torch

from conftest import tiny_levels
from oracle import mc, siren

pytestmark = pytest.mark.gpu


def _models(sds, precision="fp32"):
    from mplicits_gb300.model import SIREN
    out = []
    for sd in sds:
        m = SIREN(3, 1, [32, 32, 32], w0=30, delay_init=True, precision=precision)
        m.load_state_dict({k: torch.as_tensor(v) for k, v in sd.items()})
        out.append(m.cuda().eval())
    return out


def test_banded_volume_and_bands_match_reference(lib):
    from mplicits_gb300.meshing import BandedReconstruction
    _, sds, d = tiny_levels()
    N = int(d["N"])
    deltas = [float(x) for x in d["deltas"]]
    rec = BandedReconstruction(_models(sds), deltas, N, "cuda")
    S = rec.sample().cpu().numpy()
    assert np.abs(S - d["S_banded"]).max() <= 1e-5
    grid = siren.grid_coords(N, 2.0 / (N - 1))
    sizes = rec.band_sizes()
    for i in (1, 2):
        idx = rec.band_index[i - 1][:sizes[i - 1]].cpu().numpy()
        got = {tuple(r) for r in grid[idx].tolist()}
        ref = {tuple(r) for r in d[f"band{i}_pts"].tolist()}
        assert got == ref


def test_unculled_volume_matches_reference(lib):
    from mplicits_gb300.meshing import BandedReconstruction
    _, sds, d = tiny_levels()
    N = int(d["N"])
    rec = BandedReconstruction(_models(sds), [], N, "cuda")
    S = rec.sample().cpu().numpy()
    assert np.abs(S - d["S_full"]).max() <= 1e-5


def test_create_mesh_multistage_drop_in(lib, tmp_path):
    from mplicits_gb300.meshing import create_mesh_multistage
    _, sds, d = tiny_levels()
    N = int(d["N"])
    deltas = [float(x) for x in d["deltas"]]
    path = os.path.join(tmp_path, "m.ply")
    verts, faces, normals, values, t = create_mesh_multistage(
        _models(sds), deltas, filename=path, N=N, max_batch=32 ** 3, device="cuda",
        silent=True)
    assert t > 0 and verts.shape[0] > 0
    # the mesh is the oracle's marching cubes of the GPU volume, bit for bit
    from mplicits_gb300.meshing import BandedReconstruction
    rec = BandedReconstruction(_models(sds), deltas, N, "cuda")
    S = rec.sample().cpu().numpy().reshape(N, N, N)
    v2, f2, n2, _ = mc.marching_cubes_raw(S, 0.0, np.float32(2.0 / (N - 1)), (-1, -1, -1))
    assert np.array_equal(verts, v2) and np.array_equal(faces, f2)
    with open(path, "rb") as fh:
        head = fh.read(200)
    assert head.startswith(b"ply\nformat binary_little_endian 1.0\nelement vertex ")
