"""The reference renderer's checkpoint formats.

* ``.bin`` pairs: ``<stem>_weights.bin`` and ``<stem>_biases.bin``, flat
  little-endian float32 with no header: every nn.Linear weight row-major
  ([out, in]), layer after layer, then every bias (renderer/README.md,
  "Checkpoint format"; renderer/scripts/weights_biases_from_pth.py).
* ``.exp`` experiment descriptors: ``key = value`` lines naming, per level of
  detail 0..2 (coarse, medium, fine), the number of hidden GEMMs, the hidden
  width and the two ``.bin`` files, plus render flags
  (renderer/cuda/state.cu:662-712 reads them; renderer/scripts/
  export_experiment.py writes them).

``export_experiment`` writes the same bytes and lines as the reference's
exporter; ``load_experiment`` builds the three ``mplicits_gb300.SIREN`` levels
a descriptor names, ready for the band-culled evaluator and the tracer.
"""

from __future__ import annotations

import os
import warnings

import numpy as np
import torch

STAGES = ("coarse", "medium", "fine")
_INT_KEYS = {"lod0_layers", "lod0_hidden", "lod1_layers", "lod1_hidden", "lod2_layers",
             "lod2_hidden", "textures_layers", "textures_hidden", "surface_w0", "textures_w0"}
_BOOL_KEYS = {"is3d", "swap_y_and_z", "invert_z", "flip_y"}
_PATH_KEYS = {f"{p}_{k}" for p in ("lod0", "lod1", "lod2", "textures")
              for k in ("weights", "biases")}


def _tensors(sd_or_model):
    sd = sd_or_model.state_dict() if hasattr(sd_or_model, "state_dict") else sd_or_model
    if isinstance(sd, dict) and "model_state_dict" in sd:
        sd = sd["model_state_dict"]
    return [torch.as_tensor(v).detach().cpu().float() for v in sd.values()]


def hidden_gemms(sd_or_model):
    """(hidden width, number of hidden x hidden layers): the architecture a
    descriptor records for a level."""
    t = _tensors(sd_or_model)
    hidden = int(t[0].shape[0])
    n = sum(1 for w in t[2:-2:2] if tuple(w.shape) == (hidden, hidden))
    return hidden, n


def write_bin_pair(sd_or_model, weights_path, biases_path):
    t = _tensors(sd_or_model)
    w = np.concatenate([t[i].numpy().reshape(-1) for i in range(0, len(t), 2)])
    b = np.concatenate([t[i + 1].numpy().reshape(-1) for i in range(0, len(t), 2)])
    with open(weights_path, "wb") as f:
        f.write(w.astype("<f4").tobytes())
    with open(biases_path, "wb") as f:
        f.write(b.astype("<f4").tobytes())


def read_bin_pair(weights_path, biases_path, hidden, n_hidden_gemms, n_in=3, n_out=1):
    """State dict (``net.{i}.0.weight|bias``) of the level a ``.bin`` pair
    holds: n_in -> hidden, n_hidden_gemms x (hidden -> hidden), hidden -> n_out."""
    dims = [n_in] + [hidden] * (n_hidden_gemms + 1) + [n_out]
    w = np.fromfile(weights_path, dtype="<f4")
    b = np.fromfile(biases_path, dtype="<f4")
    nw = sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))
    nb = sum(dims[1:])
    if w.size != nw or b.size != nb:
        raise ValueError(f"{weights_path}: {w.size} weights / {b.size} biases, expected {nw} / "
                         f"{nb} for width {hidden} with {n_hidden_gemms} hidden GEMMs")
    sd, ow, ob = {}, 0, 0
    for i in range(len(dims) - 1):
        o, k = dims[i + 1], dims[i]
        sd[f"net.{i}.0.weight"] = torch.from_numpy(w[ow:ow + o * k].reshape(o, k).copy())
        sd[f"net.{i}.0.bias"] = torch.from_numpy(b[ob:ob + o].copy())
        ow += o * k
        ob += o
    return sd


def read_experiment(path):
    """The descriptor as a dict, with the renderer's defaults (is3d true,
    surface_w0 1, textures_w0 0).  Unknown keys are ignored with a warning;
    the three levels must be present (the renderer refuses otherwise)."""
    if not os.path.exists(path):
        raise FileNotFoundError(f"cannot open experiment file '{path}'")
    e = {"is3d": True, "surface_w0": 1, "textures_w0": 0}
    with open(path, encoding="utf-8") as f:
        for raw in f:
            line = raw.strip()
            if not line or line.startswith("#") or "=" not in line:
                continue
            k, v = (s.strip() for s in line.split("=", 1))
            if k in _INT_KEYS:
                e[k] = int(v)
            elif k in _BOOL_KEYS:
                e[k] = int(v) != 0
            elif k in _PATH_KEYS:
                e[k] = v
            else:
                warnings.warn(f"experiment file: unknown key '{k}' ignored")
    if not all(e.get(f"lod{i}_weights") for i in range(3)):
        raise ValueError(f"experiment file '{path}' must define lod0, lod1 and lod2 "
                         "(coarse, medium, fine)")
    return e


def export_experiment(levels, out_dir, name, data_root="data", w0=1, flip_y=False,
                      swap_y_and_z=False, invert_z=False, source=None):
    """Writes ``<name>_<stage>_{weights,biases}.bin`` for the three levels
    (models or state dicts, omega baked as the released checkpoints store
    it) and the descriptor ``<name>.exp`` into ``out_dir``; returns its path.
    ``source`` is the folder named in the descriptor's comment line."""
    if len(levels) != 3:
        raise ValueError("a descriptor holds exactly three levels (coarse, medium, fine)")
    os.makedirs(out_dir, exist_ok=True)
    rel = os.path.basename(os.path.normpath(out_dir))
    lines = [f"# exported from {source if source is not None else os.path.abspath(out_dir)}"]
    for lod, (stage, level) in enumerate(zip(STAGES, levels)):
        stem = f"{name}_{stage}"
        write_bin_pair(level, os.path.join(out_dir, stem + "_weights.bin"),
                       os.path.join(out_dir, stem + "_biases.bin"))
        hidden, n = hidden_gemms(level)
        lines += [f"lod{lod}_layers = {n}", f"lod{lod}_hidden = {hidden}",
                  f"lod{lod}_weights = {data_root}/{rel}/{stem}_weights.bin",
                  f"lod{lod}_biases = {data_root}/{rel}/{stem}_biases.bin"]
    lines += ["textures_layers = 0", "is3d = 1", f"surface_w0 = {int(w0)}", "textures_w0 = 0",
              f"swap_y_and_z = {int(swap_y_and_z)}", f"invert_z = {int(invert_z)}",
              f"flip_y = {int(flip_y)}"]
    path = os.path.join(out_dir, name + ".exp")
    with open(path, "w", encoding="utf-8") as f:
        f.write("\n".join(lines) + "\n")
    return path


def load_experiment(path, base_dir=".", device="cuda", precision="fp32"):
    """The three SIREN levels a descriptor names (paths resolved against
    ``base_dir``, the renderer's working directory), with the descriptor's
    surface_w0 as omega, and the descriptor itself."""
    from .model import SIREN
    e = read_experiment(path)
    models = []
    for lod in range(3):
        hidden, n = e[f"lod{lod}_hidden"], e[f"lod{lod}_layers"]
        sd = read_bin_pair(os.path.join(base_dir, e[f"lod{lod}_weights"]),
                           os.path.join(base_dir, e[f"lod{lod}_biases"]), hidden, n)
        m = SIREN(3, 1, [hidden] * (n + 1), w0=e["surface_w0"], delay_init=True,
                  precision=precision)
        m.load_state_dict(sd)
        models.append(m.to(device).eval())
    return models, e
