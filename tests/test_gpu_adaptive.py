"""Adaptive band widths (reconstruct.py:18-33) on the GPU: the partial sums
from the level kernels, each chunk's max |S| reduced on the device
(mpl_abs_max), one host read; against the reference's own output and the
oracle."""

import ctypes
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, golden, tiny_levels

pytestmark = pytest.mark.gpu


def _models(sds, width, precision="fp32"):
    from mplicits_gb300.model import SIREN
    out = []
    for sd in sds:
        m = SIREN(3, 1, [width] * 3, w0=30, delay_init=True, precision=precision)
        m.load_state_dict({k: torch.as_tensor(v) for k, v in sd.items()})
        out.append(m.cuda().eval())
    return out


def _write_cloud(path, pts):
    from mplicits_gb300.meshing import save_ply
    save_ply(pts, np.zeros((0, 3), np.int32), path)


def test_adaptive_deltas_match_the_reference(lib, tmp_path):
    """The reference's adaptive_deltas on the tiny three-level model, read
    from a PLY file as the CLI does, in several chunks and in one."""
    from mplicits_gb300.reconstruct import adaptive_deltas
    _, sds, _ = tiny_levels()
    g = golden("adaptive_deltas.npz")
    path = os.path.join(tmp_path, "cloud.ply")
    _write_cloud(path, g["points"])
    models = _models(sds, 32)
    for batch in (4096, 2 ** 18):
        got = adaptive_deltas(models, path, "cuda", batch=batch)
        ref = g[f"deltas_batch{batch}"]
        # each partial sum is an FP32 SDF value within 1e-5 of the reference's
        assert np.abs(np.asarray(got) - ref).max() <= 1.3e-5, (batch, got, ref)


@pytest.mark.parametrize("precision,tol", [("fp32", 1.3e-5), ("bf16", 1.3 * 2e-3)])
def test_adaptive_deltas_trained_model_vs_oracle(lib, precision, tol):
    """The trained 256-wide three-level model on 50,000 noisy surface
    samples, against the float32 numpy oracle (the BF16 bound is the
    tensor-core error of a partial sum)."""
    from mplicits_gb300.reconstruct import adaptive_deltas
    from mplicits_gb300.synthetic import surface_points
    from oracle import siren
    d = np.load(os.path.join(GOLDEN, "three_level_sphere.npz"))
    sds = [{k[3:]: d[k] for k in d.files if k.startswith(f"L{i}.")} for i in range(3)]
    pts, _ = surface_points(50000, np.random.default_rng(4), noise=0.002)
    got = adaptive_deltas(_models(sds, 256, precision), pts, "cuda", batch=2 ** 14)
    levels = [([(sd[f"net.{j}.0.weight"], sd[f"net.{j}.0.bias"]) for j in range(4)],
               [30.0, 30.0, 30.0]) for sd in sds]
    ref = siren.adaptive_deltas(levels, pts, batch=2 ** 14)
    assert np.abs(np.asarray(got) - np.asarray(ref)).max() <= tol, (got, ref)


def test_abs_max_is_the_exact_maximum(lib):
    """mpl_abs_max equals torch's max |S| bit for bit (signed zeros, the
    largest and smallest finite values, tails not a multiple of the block),
    is NaN when an element is NaN, and 0 for an empty input."""
    from mplicits_gb300 import capi
    out = torch.full((1,), -1.0, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(3)
    for n in (1, 31, 257, 100003, 3 << 20):
        S = torch.randn(n, device="cuda", generator=g) * 10 ** torch.randint(
            -30, 30, (n,), device="cuda", generator=g).float()
        S[0] = -0.0
        capi.check(lib.mpl_abs_max(capi.ptr(S), n, capi.ptr(out), capi.stream_ptr()), "abs_max")
        assert torch.equal(out[0], S.abs().max()), n
    big = float(np.finfo(np.float32).max)
    S = torch.tensor([1.0, -big, 2.0], device="cuda")
    capi.check(lib.mpl_abs_max(capi.ptr(S), 3, capi.ptr(out), capi.stream_ptr()), "abs_max")
    assert out.item() == big
    S[1] = float("nan")
    capi.check(lib.mpl_abs_max(capi.ptr(S), 3, capi.ptr(out), capi.stream_ptr()), "abs_max")
    assert torch.isnan(out).item()
    capi.check(lib.mpl_abs_max(None, 0, capi.ptr(out), capi.stream_ptr()), "abs_max")
    assert out.item() == 0.0
    assert lib.mpl_abs_max(None, 5, capi.ptr(out), capi.stream_ptr()) == capi.MPL_ERR_INVALID_ARG


def test_adaptive_deltas_skip_a_nan_chunk_like_the_reference(lib):
    """reconstruct.py's ``worst = max(worst, float(s.abs().max()))`` keeps
    ``worst`` when a chunk's maximum is NaN; a point with a NaN coordinate
    therefore drops its whole chunk from the band width."""
    from mplicits_gb300.reconstruct import adaptive_deltas
    from oracle import siren
    levels, sds, _ = tiny_levels()
    pts = golden("adaptive_deltas.npz")["points"][:3000].copy()
    pts[1500, 1] = np.nan
    got = adaptive_deltas(_models(sds, 32), pts, "cuda", batch=1000)
    ref = siren.adaptive_deltas(levels, np.concatenate([pts[:1000], pts[2000:]]), batch=1000)
    assert np.abs(np.asarray(got) - np.asarray(ref)).max() <= 1.3e-5


def test_reconstruct_cli_input_uses_adaptive_deltas(lib, tmp_path, capsys):
    """reconstruct.py --multistage --input: the printed band widths are
    adaptive_deltas of the cloud, and the mesh is the banded reconstruction
    with them."""
    from mplicits_gb300.meshing import BandedReconstruction
    from mplicits_gb300.reconstruct import adaptive_deltas, main
    _, sds, _ = tiny_levels()
    models = _models(sds, 32)
    # the trainers save the coarser levels with omega baked in, and the CLI
    # loads --coarse_path and --medium_path with w0 = 1 (reconstruct.py:99-112)
    models[0].update_omegas(w0=1)
    models[1].update_omegas(w0=1)
    paths = []
    for name, m in zip(("coarse", "medium", "fine"), models):
        p = os.path.join(tmp_path, f"{name}.pth")
        torch.save({k: v.cpu() for k, v in m.state_dict().items()}, p)
        paths.append(p)
    # points near the zero set of f0 + f1, so the bands are narrow
    g = golden("adaptive_deltas.npz")
    x = torch.from_numpy(g["points"]).cuda()
    with torch.no_grad():
        s01 = (models[0](x)["model_out"] + models[1](x)["model_out"]).squeeze(-1)
    keep = torch.argsort(s01.abs())[:2000].cpu().numpy()
    cloud = os.path.join(tmp_path, "cloud.ply")
    _write_cloud(cloud, g["points"][keep])
    out = os.path.join(tmp_path, "out.ply")
    main([paths[2], out, "--coarse_path", paths[0], "--medium_path", paths[1], "--w0", "30",
          "-r", "48", "--device", "cuda", "--multistage", "--input", cloud])
    text = capsys.readouterr().out
    line = next(l for l in text.splitlines() if l.startswith("adaptive band widths"))
    printed = [float(v) for v in line.split(":", 1)[1].split(",")]
    deltas = adaptive_deltas(models, cloud, "cuda")
    assert np.allclose(printed, deltas, rtol=1e-3, atol=0)
    assert "SAMPLING_TIME_S:" in text
    # the CLI's chunks are 32^3 points (reconstruct.py:128), which matters
    # when the widths grow
    rec = BandedReconstruction(models, deltas, 48, "cuda", chunk=32 ** 3)
    rec.sample()
    verts, faces, _, _ = rec.mesh()
    head = open(out, "rb").read().split(b"end_header\n")[0].decode()
    assert f"element vertex {verts.shape[0]}" in head
    assert f"element face {faces.shape[0]}" in head
