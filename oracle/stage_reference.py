"""CHECKER INFRASTRUCTURE (oracle): stage the reference's C sources for the
oracle build and the reference arm of bench.py.

    python oracle/stage_reference.py SRC_DIR     (or DISCO_REFERENCE=SRC_DIR)

copies the reference's C sources and headers (every *.c / *.h, keeping the
directory layout) from SRC_DIR into baseline/_ref/src.  That folder is
git-ignored (it is never committed) but travels with the working tree, so
oracle/ref/Makefile can build the unmodified reference on a machine where
SRC_DIR does not exist.  Nothing is edited: the copy is byte for byte.
"""
from __future__ import annotations

import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STAGED = os.path.join(ROOT, "baseline", "_ref", "src")


def stage(src: str) -> str:
    if not os.path.isfile(os.path.join(src, "paul.h")):
        raise SystemExit(f"{src}: not the reference source tree (no paul.h)")
    n = 0
    for dp, dns, fns in os.walk(src):
        dns[:] = [d for d in dns if not d.startswith(".")]
        for fn in fns:
            if not fn.endswith((".c", ".h")):
                continue
            rel = os.path.relpath(os.path.join(dp, fn), src)
            dst = os.path.join(STAGED, rel)
            os.makedirs(os.path.dirname(dst), exist_ok=True)
            shutil.copyfile(os.path.join(dp, fn), dst)
            n += 1
    print(f"staged {n} files into {STAGED}")
    return STAGED


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DISCO_REFERENCE")
    if not src:
        raise SystemExit("usage: python oracle/stage_reference.py SRC_DIR (or set DISCO_REFERENCE)")
    stage(src)
