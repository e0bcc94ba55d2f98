"""Golden output of the reference's renderer exporter.

    python tests/golden/make_export_golden.py --ref <reference checkout>

Writes the three levels of tests/golden/tiny_three_level.npz as
results/tiny/{coarse,medium,fine}/best.pth in a temporary folder, runs the
reference's own renderer/scripts/export_experiment.py on it (from a
reference checkout, ``--ref`` or ``MPLICITS_REFERENCE``), and stores the .bin pairs and
the .exp descriptor it wrote under tests/golden/export_experiment/.  The
descriptor's first line names the absolute results folder; the fixture keeps
the relative name the script was given, so the line is reproducible.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile

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
    d = np.load(os.path.join(HERE, "tiny_three_level.npz"))
    out_dir = os.path.join(HERE, "export_experiment")
    os.makedirs(out_dir, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        for i, stage in enumerate(("coarse", "medium", "fine")):
            sd = {}
            for j in range(4):
                sd[f"net.{j}.0.weight"] = torch.from_numpy(d[f"L{i}.net.{j}.0.weight"])
                sd[f"net.{j}.0.bias"] = torch.from_numpy(d[f"L{i}.net.{j}.0.bias"])
            os.makedirs(os.path.join(tmp, "results", "tiny", stage))
            torch.save(sd, os.path.join(tmp, "results", "tiny", stage, "best.pth"))
        subprocess.run([sys.executable, os.path.join(REF, "renderer", "scripts",
                                                     "export_experiment.py"),
                        "results/tiny", "--out", "released", "--flip-y"], cwd=tmp, check=True)
        for f in sorted(os.listdir(os.path.join(tmp, "released"))):
            shutil.copy(os.path.join(tmp, "released", f), os.path.join(out_dir, f))
        # the first line holds the temporary absolute path
        exp = os.path.join(out_dir, "tiny.exp")
        lines = open(exp).read().splitlines()
        lines[0] = "# exported from results/tiny"
        open(exp, "w").write("\n".join(lines) + "\n")
    print("written", out_dir)


if __name__ == "__main__":
    main()
