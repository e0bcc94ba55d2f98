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


def _trained_levels(precision):
    from mplicits_gb300.model import SIREN
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "three_level_sphere.npz"))
    out = []
    for i in range(3):
        sd = {k[3:]: d[k] for k in d.files if k.startswith(f"L{i}.")}
        m = SIREN(3, 1, [256, 256, 256], w0=30, delay_init=True, precision=precision)
        m.load_state_dict({k: torch.from_numpy(v) for k, v in sd.items()})
        out.append(m.cuda().eval())
    return out


@pytest.mark.parametrize("precision,margin", [("bf16", 2e-3), ("fp16", 1e-3)])
def test_refined_tensor_core_bands_and_mesh_topology_equal_fp32(lib, precision, margin):
    """With the FP32 re-evaluation margin, the tensor-core pipeline cuts the
    same band lists as the plain FP32 pipeline and its marching cubes sees the
    same signs (identical face arrays) on the trained three-level model."""
    from mplicits_gb300.meshing import BandedReconstruction
    N, deltas = 128, [0.05, 0.01]
    ref = BandedReconstruction(_trained_levels("fp32"), deltas, N, "cuda")
    ref.sample()
    rec = BandedReconstruction(_trained_levels(precision), deltas, N, "cuda", precision,
                               refine_margin=margin)
    rec.sample()
    for i in range(2):
        a = np.sort(ref.band_index[i][:ref.band_sizes()[i]].cpu().numpy())
        b = np.sort(rec.band_index[i][:rec.band_sizes()[i]].cpu().numpy())
        assert np.array_equal(a, b), i
    va, fa, _, _ = ref.mesh()
    vb, fb, _, _ = rec.mesh()
    assert torch.equal(fa, fb)
    # vertices with an end within the margin are FP32; the rest carry the
    # tensor-core error only
    assert (va - vb).abs().max().item() < 2.0 / (N - 1)
    S32, S16 = ref.S.cpu().numpy(), rec.S.cpu().numpy()
    near = np.abs(S16) < margin  # the points the zero-level pass recomputed in FP32
    assert near.any() and np.array_equal(S32[near], S16[near])


def test_create_mesh_single_level_drop_in(lib, tmp_path):
    """create_mesh (i3d/meshing.py:72-132): one level on the whole grid, then
    marching cubes.  The volume is within 1e-5 of the oracle's float32
    evaluation, and the mesh is the oracle's marching cubes of the GPU
    volume bit for bit; the PLY holds that mesh."""
    from mplicits_gb300.meshing import BandedReconstruction, create_mesh
    levels, sds, d = tiny_levels()
    N = 40
    path = os.path.join(tmp_path, "single.ply")
    model = _models(sds)[0]
    verts, faces, normals, values = create_mesh(model, filename=path, N=N, device="cuda",
                                                silent=True)
    rec = BandedReconstruction([model], [], N, "cuda")
    S = rec.sample().cpu().numpy()
    ref, _ = siren.multistage_sdf(levels[:1], [], N)
    assert np.abs(S - ref).max() <= 1e-5
    v2, f2, n2, val2 = mc.marching_cubes_raw(S.reshape(N, N, N), 0.0, np.float32(2.0 / (N - 1)),
                                             (-1, -1, -1))
    assert verts.shape[0] > 100
    for a, b in ((verts, v2), (faces, f2), (normals, n2), (values, val2)):
        assert np.array_equal(a, b)
    head = open(path, "rb").read().split(b"end_header\n")[0].decode()
    assert f"element vertex {verts.shape[0]}" in head and f"element face {faces.shape[0]}" in head


def test_growing_band_widths_match_reference(lib):
    """Band widths that grow (0.005 then 0.05) over chunks of 37 points: the
    reference's masks cover whole chunks, and 10 chunks stop after level 0.
    The volume is within 1e-5 of the reference's, and each residual level
    evaluated exactly the reference's points."""
    from mplicits_gb300.meshing import BandedReconstruction, create_mesh_multistage
    _, sds, _ = tiny_levels()
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "multistage_increasing.npz"))
    N, chunk = int(g["N"]), int(g["chunk"])
    deltas = [float(x) for x in g["deltas"]]
    rec = BandedReconstruction(_models(sds), deltas, N, "cuda", chunk=chunk)
    assert not rec.nested
    S = rec.sample().cpu().numpy()
    assert np.abs(S - g["S"]).max() <= 1e-5
    grid = siren.grid_coords(N, 2.0 / (N - 1))
    sizes = rec.band_sizes()
    for i in (1, 2):
        idx = rec.band_index[i - 1][:sizes[i - 1]].cpu().numpy()
        assert idx.shape[0] == g[f"band{i}_pts"].shape[0], i
        got = {tuple(r) for r in grid[idx].tolist()}
        ref = {tuple(r) for r in g[f"band{i}_pts"].tolist()}
        assert got == ref, i
    # the drop-in passes max_batch through as the chunk
    verts, faces, _, _, _ = create_mesh_multistage(_models(sds), deltas, N=N, max_batch=chunk,
                                                   device="cuda", silent=True)
    v2, f2, _, _ = mc.marching_cubes_raw(S.reshape(N, N, N), 0.0, np.float32(2.0 / (N - 1)),
                                         (-1, -1, -1))
    assert np.array_equal(faces, f2) and np.array_equal(verts, v2)
