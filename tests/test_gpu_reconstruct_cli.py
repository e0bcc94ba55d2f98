"""The reconstruct.py drop-in end to end: three level checkpoints written
with torch.save, the reference's positional arguments and flags, the
SAMPLING_TIME_S line that reproduce.py parses, and a PLY whose mesh is the
one BandedReconstruction gives for the same levels."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _levels():
    from mplicits_gb300.model import SIREN
    out = []
    for seed, scale in ((0, 1.0), (1, 0.1), (2, 0.02)):
        torch.manual_seed(seed)
        m = SIREN(3, 1, [128, 128, 128], w0=30)
        with torch.no_grad():
            m.net[-1][0].weight.mul_(scale)
            m.net[-1][0].bias.mul_(scale)
        out.append(m)
    return out


def _ply_counts(path):
    data = open(path, "rb").read()
    head = data[:data.index(b"end_header\n")].decode("ascii").splitlines()
    nv = int(next(l for l in head if l.startswith("element vertex")).split()[-1])
    nf = int(next(l for l in head if l.startswith("element face")).split()[-1])
    return nv, nf


@pytest.mark.parametrize("precision", ["fp32", "bf16"])
def test_reconstruct_cli_multistage(lib, tmp_path, capsys, precision):
    from mplicits_gb300.meshing import BandedReconstruction
    from mplicits_gb300.reconstruct import main
    coarse, medium, fine = _levels()
    # the trainers save the coarser levels with omega baked in (loaded with w0 = 1)
    coarse.update_omegas(w0=1)
    medium.update_omegas(w0=1)
    paths = []
    for name, m in (("coarse", coarse), ("medium", medium), ("fine", fine)):
        p = tmp_path / f"{name}.pth"
        torch.save(m.state_dict(), p)
        paths.append(str(p))
    out = tmp_path / "mesh" / "out.ply"
    N, deltas = 64, [0.05, 0.02]
    main([paths[2], str(out), "--coarse_path", paths[0], "--medium_path", paths[1], "--w0", "30",
          "-r", str(N), "--device", "cuda", "--multistage", "--deltas", *map(str, deltas),
          "--precision", precision])
    text = capsys.readouterr().out
    line = next(l for l in text.splitlines() if l.startswith("SAMPLING_TIME_S:"))
    assert float(line.split(":", 1)[1]) > 0
    nv, nf = _ply_counts(out)
    levels = [m.cuda().eval() for m in (coarse, medium, fine)]
    rec = BandedReconstruction(levels, deltas, N, "cuda", precision)
    rec.sample()
    verts, faces, _, _ = rec.mesh()
    assert nv == verts.shape[0] > 100 and nf == faces.shape[0]
