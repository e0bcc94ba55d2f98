"""The renderer checkpoint formats against the reference exporter's own
output (tests/golden/export_experiment, made by make_export_golden.py)."""

import os
import warnings

import numpy as np
import pytest
import torch

from conftest import tiny_levels

GOLD = os.path.join(os.path.dirname(__file__), "golden", "export_experiment")


def _sds():
    _, sds, _ = tiny_levels()
    return [{k: torch.from_numpy(v) for k, v in sd.items()} for sd in sds]


def test_export_matches_reference_exporter_byte_for_byte(tmp_path):
    from mplicits_gb300.formats import export_experiment
    out = os.path.join(tmp_path, "released")
    path = export_experiment(_sds(), out, "tiny", flip_y=True, source="results/tiny")
    for f in sorted(os.listdir(GOLD)):
        with open(os.path.join(GOLD, f), "rb") as a, open(os.path.join(out, f), "rb") as b:
            assert a.read() == b.read(), f
    assert os.path.basename(path) == "tiny.exp"


def test_read_descriptor_and_bins_reproduce_the_levels():
    from mplicits_gb300.formats import read_bin_pair, read_experiment
    e = read_experiment(os.path.join(GOLD, "tiny.exp"))
    assert e["flip_y"] and e["is3d"] and e["surface_w0"] == 1 and not e["swap_y_and_z"]
    for lod, sd in enumerate(_sds()):
        assert (e[f"lod{lod}_hidden"], e[f"lod{lod}_layers"]) == (32, 2)
        stem = os.path.basename(e[f"lod{lod}_weights"])
        got = read_bin_pair(os.path.join(GOLD, stem),
                            os.path.join(GOLD, stem.replace("_weights", "_biases")), 32, 2)
        assert list(got) == list(sd)
        for k in sd:
            assert torch.equal(got[k], sd[k])


def test_round_trip_wide_level_and_loader(tmp_path):
    from mplicits_gb300.formats import export_experiment, load_experiment
    from mplicits_gb300.model import SIREN
    torch.manual_seed(3)
    levels = [SIREN(3, 1, [w] * 3, w0=30) for w in (256, 128, 64)]
    for m in levels:
        m.update_omegas(w0=1)  # omega baked, as the released checkpoints store it
    out = os.path.join(tmp_path, "data", "mine")
    export_experiment(levels, out, "m", data_root="data", w0=1)
    models, e = load_experiment(os.path.join(out, "m.exp"), base_dir=str(tmp_path), device="cpu")
    for a, b in zip(levels, models):
        assert b.omegas() == [1.0, 1.0, 1.0]
        for (ka, va), (kb, vb) in zip(a.state_dict().items(), b.state_dict().items()):
            assert ka == kb and torch.equal(va, vb)


def test_descriptor_errors(tmp_path):
    from mplicits_gb300.formats import read_bin_pair, read_experiment
    p = os.path.join(tmp_path, "bad.exp")
    with open(p, "w") as f:
        f.write("lod0_weights = a.bin\nlod1_weights = b.bin\nmystery = 3\n")
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        with pytest.raises(ValueError):
            read_experiment(p)
        assert any("mystery" in str(x.message) for x in w)
    with pytest.raises(FileNotFoundError):
        read_experiment(os.path.join(tmp_path, "none.exp"))
    with pytest.raises(ValueError):
        read_bin_pair(os.path.join(GOLD, "tiny_coarse_weights.bin"),
                      os.path.join(GOLD, "tiny_coarse_biases.bin"), 32, 3)
