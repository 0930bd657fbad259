"""Copies the reference MFEM sources that oracle/ref/Makefile compiles
(general/, linalg/, mesh/, fem/, the config/ headers and mfem.hpp) into
baseline/_ref/src/, a git-ignored folder that travels with the working tree to
the GPU host, where build() compiles them for that host's CPU. The copy is an
unmodified subset of the reference tree, used only to build the reference's own
CPU partial-assembly path for the CPU baseline; nothing of it is committed.

    python oracle/ref/stage_reference.py <reference source tree>
    (or set MFEM_REFERENCE_DIR)
"""
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
DEST = os.path.join(REPO, "baseline", "_ref", "src")
DIRS = ("general", "linalg", "mesh", "fem")
TOP = ("mfem.hpp",)


def stage(ref, dest=DEST):
    if not os.path.exists(os.path.join(ref, "mfem.hpp")):
        raise SystemExit(f"{ref} is not an MFEM source tree (no mfem.hpp)")
    if os.path.isdir(dest):
        shutil.rmtree(dest)
    os.makedirs(dest)
    keep = (".cpp", ".hpp", ".h", ".inc")
    for d in DIRS:
        shutil.copytree(os.path.join(ref, d), os.path.join(dest, d),
                        ignore=lambda src, names: [n for n in names
                                                   if os.path.isfile(os.path.join(src, n))
                                                   and not n.endswith(keep)])
    os.makedirs(os.path.join(dest, "config"))
    for f in os.listdir(os.path.join(ref, "config")):
        if f.endswith(".hpp"):
            shutil.copy2(os.path.join(ref, "config", f), os.path.join(dest, "config", f))
    for f in TOP:
        shutil.copy2(os.path.join(ref, f), os.path.join(dest, f))
    return dest


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MFEM_REFERENCE_DIR")
    if not ref:
        raise SystemExit("usage: stage_reference.py <reference source tree> (or MFEM_REFERENCE_DIR)")
    print(stage(ref))
