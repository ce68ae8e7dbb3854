"""Where the fixture scripts find the reference checkout (sgl_analytic v0.2.0).

The scripts in this directory run the reference's own code to make golden vectors; they are run
by hand in a development container that holds the reference source, never by the tests.  The
checkout is named by ``--reference PATH`` or the ``SGL_REFERENCE`` environment variable: the
directory that holds ``src/sgl_analytic`` and ``tests/reference``.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path


def reference_root(argv=None) -> Path:
    argv = sys.argv if argv is None else argv
    path = None
    for i, a in enumerate(argv):
        if a == "--reference" and i + 1 < len(argv):
            path = argv[i + 1]
        elif a.startswith("--reference="):
            path = a.split("=", 1)[1]
    path = path or os.environ.get("SGL_REFERENCE")
    if not path:
        raise SystemExit("name the reference checkout: --reference PATH or SGL_REFERENCE=PATH "
                         "(the directory holding src/sgl_analytic)")
    root = Path(path).resolve()
    if not (root / "src" / "sgl_analytic").is_dir():
        raise SystemExit(f"{root} does not hold src/sgl_analytic")
    return root


def strip_reference_args(argv):
    """argv without the --reference option (for scripts that parse their own arguments)."""
    out, skip = [], False
    for a in argv:
        if skip:
            skip = False
            continue
        if a == "--reference":
            skip = True
            continue
        if a.startswith("--reference="):
            continue
        out.append(a)
    return out
