"""Checkpoint loaders against files the reference wrote (i3d/util.py:79-142,
i3d/model.py:322-424), and the oracle's adaptive band widths against the
reference's adaptive_deltas (reconstruct.py:18-33).  Fixtures from
tests/golden/make_loader_golden.py; the CPU tests load only (no kernels)."""

import os
import shutil

import numpy as np
import pytest
import torch

from conftest import GOLDEN, golden, tiny_levels


def _copy(tmp_path, name):
    dst = os.path.join(tmp_path, name)
    shutil.copy(os.path.join(GOLDEN, name), dst)
    return dst


def test_from_pth_loads_a_reference_checkpoint(tmp_path):
    from mplicits_gb300.model import SIREN, from_pth
    path = _copy(tmp_path, "ref_siren_w64.pth")
    ref = torch.load(path)
    m = from_pth(path, w0=30)
    assert isinstance(m, SIREN)
    assert [l.out_features for l in m.linears()] == [64, 64, 1]
    assert m.omegas() == [30.0, 30.0]
    sd = m.state_dict()
    assert list(sd.keys()) == list(ref.keys())
    for k in ref:
        assert torch.equal(sd[k], ref[k])
    assert not os.path.exists(os.path.join(tmp_path, "ref_siren_w64_v2.pth"))


def test_from_pth_upgrades_v1_keys_like_the_reference(tmp_path, capsys):
    """A state_dict of the old SIREN class (net.net.* keys) loads after the
    key upgrade, and the upgraded file written beside it holds what the
    reference's from_pth wrote: the same keys in the same order, the same
    tensors."""
    from mplicits_gb300.model import from_pth
    path = _copy(tmp_path, "ref_siren_w64_v1.pth")
    m = from_pth(path, w0=30)
    assert "Found weights from old version of SIREN" in capsys.readouterr().out
    g = golden("loaders.npz")
    v2 = torch.load(os.path.join(tmp_path, "ref_siren_w64_v1_v2.pth"))
    assert list(v2.keys()) == [str(k) for k in g["v2_keys"]]
    for k, v in v2.items():
        assert np.array_equal(v.numpy(), g[f"v2.{k}"])
    ref = torch.load(os.path.join(GOLDEN, "ref_siren_w64.pth"))
    for k, v in m.state_dict().items():
        assert torch.equal(v, ref[k])


def test_from_state_dict_reports_the_upgrade():
    from mplicits_gb300.model import from_state_dict
    ref = torch.load(os.path.join(GOLDEN, "ref_siren_w64.pth"))
    _, up = from_state_dict(ref, w0=30)
    assert up is False
    v1 = type(ref)((f"net.{k}", v) for k, v in ref.items())
    m, up = from_state_dict(v1, w0=30)
    assert up is True
    assert torch.equal(m.state_dict()["net.2.0.weight"], ref["net.2.0.weight"])


def test_from_pth_missing_file_raises_like_the_reference(tmp_path):
    from mplicits_gb300.model import from_pth
    with pytest.raises(FileNotFoundError):
        from_pth(os.path.join(tmp_path, "nope.pth"))


def test_oracle_adaptive_deltas_match_the_reference():
    """The oracle's restatement of reconstruct.py:18-33 in float32 numpy
    against the reference's own function on the same points (FP32 matmul
    order differs, so the bound is that of an FP32 SDF value, times 1.3)."""
    from oracle import siren
    levels, _, _ = tiny_levels()
    g = golden("adaptive_deltas.npz")
    for batch in (4096, 2 ** 18):
        got = siren.adaptive_deltas(levels, g["points"], batch=batch)
        ref = g[f"deltas_batch{batch}"]
        assert np.abs(np.asarray(got) - ref).max() <= 1.3e-6


@pytest.mark.gpu
def test_reference_checkpoints_evaluate_like_the_reference(lib, tmp_path):
    """The loaded models run on the fused FP32 kernel and give the reference
    model's outputs on the probe points within 1e-5."""
    from mplicits_gb300.model import from_pth
    g = golden("loaders.npz")
    x = torch.from_numpy(g["probe"]).cuda()
    for name, key in (("ref_siren_w64.pth", "out"), ("ref_siren_w64_v1.pth", "out_v1")):
        m = from_pth(_copy(tmp_path, name), w0=30, device="cuda")
        with torch.no_grad():
            y = m(x)["model_out"].squeeze(-1).cpu().numpy()
        assert np.abs(y - g[key]).max() <= 1e-5, name
