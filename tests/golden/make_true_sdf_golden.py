"""Golden values of the coarse trainer's loss, ``true_sdf``
(i3d/loss_functions.py:123-163), and the parameter gradients autograd gives
for it, from the reference's own code.

    python tests/golden/make_true_sdf_golden.py --ref <reference checkout>

Imports i3d.model and i3d.loss_functions from a reference checkout (``--ref``
or ``MPLICITS_REFERENCE``); writes tests/golden/loss_true_sdf.npz.
"""

from __future__ import annotations

import os
import sys

import numpy as np
import torch

REF = None  # the reference checkout: main() sets it from --ref PATH or MPLICITS_REFERENCE


def _reference_root():
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    from refroot import reference_root
    return reference_root()
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    global REF
    REF = _reference_root()
    sys.path.insert(0, REF)
    from i3d.loss_functions import true_sdf
    from i3d.model import SIREN
    torch.manual_seed(33)
    model = SIREN(3, 1, [32, 32, 32], w0=30)
    rng = np.random.default_rng(8)
    n = 96
    x = rng.uniform(-0.8, 0.8, (n, 3)).astype(np.float32)
    normals = (x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.float32)
    sdf = np.zeros((n, 1), np.float32)
    sdf[40:, 0] = rng.uniform(-0.3, 0.3, n - 40).astype(np.float32)
    losses = true_sdf(model(torch.from_numpy(x)), {"sdf": torch.from_numpy(sdf),
                                                    "normals": torch.from_numpy(normals)})
    total = sum(losses.values())
    total.backward()
    out = {f"model.{k}": v.detach().numpy().copy() for k, v in model.state_dict().items()}
    out.update({f"grad.{k}": p.grad.numpy().copy() for k, p in model.named_parameters()})
    out.update({f"loss.{k}": np.array(float(v)) for k, v in losses.items()})
    out.update(x=x, normals=normals, sdf=sdf)
    np.savez_compressed(os.path.join(HERE, "loss_true_sdf.npz"), **out)
    print({k: float(v) for k, v in losses.items()})


if __name__ == "__main__":
    main()
