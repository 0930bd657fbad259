"""Regenerate the golden fixtures in this directory from the reference itself.

Builds the unmodified reference MFEM sources (serial CPU library) with the
recipe in oracle/ref/Makefile, runs oracle/ref/golden_driver.cpp -- which calls
MFEM's own partial-assembly path (ElementRestriction, DofToQuad, geometric
factors, PADiffusionSetup, AddMultPA, AssembleDiagonalPA, BilinearForm::Mult,
PCG + OperatorJacobiSmoother) -- and packs each case's .npy dumps into one
compressed <case>.npz here.

    python tests/golden/make_golden.py --ref <reference source tree>
    (or set MFEM_REFERENCE_DIR)

Needs the reference tree, g++ and make; it is run in the development container,
never at test time.
"""
import argparse
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MFEM_REFERENCE_DIR"),
                    help="the reference MFEM source tree (default: $MFEM_REFERENCE_DIR)")
    ap.add_argument("-j", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--cases", default=None, help="comma-separated case names to (re)write (default: all)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("the reference tree is required: --ref <path> or MFEM_REFERENCE_DIR")
    refdir = os.path.join(REPO, "oracle", "ref")
    subprocess.check_call(["make", "-C", refdir, f"REF={args.ref}", f"-j{args.j}"])
    raw = os.path.join(REPO, "oracle", "_ref", "golden_raw")
    os.makedirs(raw, exist_ok=True)
    drv = os.path.join(REPO, "oracle", "_ref", "golden_driver")
    out = subprocess.check_output([drv, raw], text=True)
    sys.stdout.write(out)
    wanted = set(args.cases.split(",")) if args.cases else None
    for case in sorted(os.listdir(raw)):
        if wanted is not None and case not in wanted:
            continue
        cdir = os.path.join(raw, case)
        arrays = {f[:-4]: np.load(os.path.join(cdir, f))
                  for f in sorted(os.listdir(cdir)) if f.endswith(".npy")}
        np.savez_compressed(os.path.join(HERE, case + ".npz"), **arrays)
        print(f"wrote {case}.npz ({len(arrays)} arrays)")


if __name__ == "__main__":
    main()
