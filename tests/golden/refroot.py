"""Location of the reference checkout for the golden-vector generators.

The generators import the reference's own code, so they need its source
tree.  Pass it as ``--ref PATH`` on the command line or in the environment
variable ``MPLICITS_REFERENCE``; nothing else is assumed.
"""

from __future__ import annotations

import os
import sys


def reference_root(argv=None):
    argv = sys.argv[1:] if argv is None else list(argv)
    root = None
    for i, a in enumerate(argv):
        if a == "--ref" and i + 1 < len(argv):
            root = argv[i + 1]
        elif a.startswith("--ref="):
            root = a.split("=", 1)[1]
    root = root or os.environ.get("MPLICITS_REFERENCE")
    if not root:
        raise SystemExit("give the reference checkout as --ref PATH or MPLICITS_REFERENCE=PATH")
    if not os.path.isdir(os.path.join(root, "i3d")):
        raise SystemExit(f"{root}: not a reference checkout (no i3d/ package)")
    return os.path.abspath(root)
