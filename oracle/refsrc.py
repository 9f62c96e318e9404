"""Where the reference simulator's sources are, for the test-infrastructure
recipes that compile them (oracle/ref_harness: its setup and gating code for
the host; oracle/ref_cuda: its CUDA RKC path for the GPU) and for the tests
that read its model files.  Nothing here is part of the product.

The location is the environment variable GBRKC_REFERENCE, else the staged
copy baseline/_ref/src.  The staged copy is git-ignored (never committed);
``python oracle/refsrc.py stage SRC`` makes it from a reference checkout at
SRC, so that the sources travel with the working tree to a machine where no
checkout is mounted (the GPU machine), as a pip-installed reference would.

    python oracle/refsrc.py stage SRC     copy the checkout at SRC
    python oracle/refsrc.py where         print the location (or nothing)
"""
from __future__ import annotations

import os
import shutil
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGED = os.path.join(ROOT, "baseline", "_ref", "src")
ENV = "GBRKC_REFERENCE"

# what a build of the reference's RKC path and its model files needs
SUFFIXES = (".cu", ".cuh", ".h", ".txt", ".csv", ".sh")


def reference_dir():
    """The reference checkout (GBRKC_REFERENCE) or its staged copy, or None."""
    env = os.environ.get(ENV)
    for d in ([env] if env else []) + [STAGED]:
        if d and os.path.isfile(os.path.join(d, "solve_rkc.cu")):
            return os.path.abspath(d)
    return None


def stage(src: str) -> str:
    """Copy the reference's sources and model files from src into the staged
    copy (replacing it).  Returns the staged directory."""
    if not os.path.isfile(os.path.join(src, "solve_rkc.cu")):
        raise SystemExit(f"{src}: not a reference checkout (no solve_rkc.cu)")
    if os.path.isdir(STAGED):
        shutil.rmtree(STAGED)
    os.makedirs(STAGED)
    for name in sorted(os.listdir(src)):
        p = os.path.join(src, name)
        if os.path.isfile(p) and (name.endswith(SUFFIXES) or name in ("Makefile", "README.txt", "LICENSE")):
            shutil.copy2(p, os.path.join(STAGED, name))
    return STAGED


if __name__ == "__main__":
    if len(sys.argv) >= 3 and sys.argv[1] == "stage":
        print(stage(sys.argv[2]))
    elif len(sys.argv) >= 2 and sys.argv[1] == "where":
        d = reference_dir()
        if d:
            print(d)
    else:
        raise SystemExit(__doc__)
