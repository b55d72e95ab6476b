"""Where the fixture generators find the reference checkout.

The generators run the reference PythonMHD itself, so they need its checkout
(the directory holding ``Source/``).  It comes from the first command-line
argument or, failing that, the ``PYTHONMHD_REFERENCE`` environment variable;
there is no default location.
"""
from __future__ import annotations

import os
import sys


def reference_root(argv=None, required=True):
    argv = sys.argv if argv is None else argv
    root = argv[1] if len(argv) > 1 else os.environ.get("PYTHONMHD_REFERENCE")
    if root is None and required:
        raise SystemExit(f"usage: python -B {argv[0]} <PythonMHD checkout> "
                         "(or set PYTHONMHD_REFERENCE)")
    if root is not None and not os.path.isdir(os.path.join(root, "Source")):
        raise SystemExit(f"{root}: not a PythonMHD checkout (no Source/ directory)")
    return root
