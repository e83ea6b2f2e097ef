"""Assemble an R source package that runs the reference's R code on this engine.

The R front-end stays the reference's own (R/RAccRQA.R calls
.C("R_double_accrqa_*") and NAMESPACE loads useDynLib(AccRQA)); only the
compiled library changes.  This script takes the R package files from a
checkout of the reference (DESCRIPTION, NAMESPACE, R/, man/, and its
testthat tests when present) and this engine's sources (the CUDA and C++
sources and the C/C++ headers), adds this engine's `configure` and
`src/Makevars.in`, and writes the result to a directory that
`R CMD INSTALL <dir>` builds for sm_103a:

    python -m accrqa_gb300.rpkg.assemble --reference <reference tree> --out <dir>
    R CMD INSTALL <dir>

Nothing of the reference is stored in this repository; the package directory
is a build output.
"""
from __future__ import annotations

import argparse
import os
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

R_FILES = ["DESCRIPTION", "NAMESPACE", "LICENSE"]
R_DIRS = ["R", "man"]


def assemble(reference: str, out: str) -> str:
    if not os.path.isfile(os.path.join(reference, "R", "RAccRQA.R")):
        raise SystemExit(f"{reference} is not an AccRQA reference tree (no R/RAccRQA.R)")
    if os.path.exists(out):
        shutil.rmtree(out)
    os.makedirs(os.path.join(out, "src"))
    for f in R_FILES:
        src = os.path.join(reference, f)
        if os.path.isfile(src):
            shutil.copy2(src, os.path.join(out, f))
    for d in R_DIRS:
        src = os.path.join(reference, d)
        if os.path.isdir(src):
            shutil.copytree(src, os.path.join(out, d))
    tests = os.path.join(reference, "tests", "testthat")
    if os.path.isdir(tests):
        shutil.copytree(tests, os.path.join(out, "tests", "testthat"))
        tt = os.path.join(reference, "tests", "testthat.R")
        if os.path.isfile(tt):
            shutil.copy2(tt, os.path.join(out, "tests", "testthat.R"))
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cpp", ".cu", ".h", ".hpp", ".cuh")):
            shutil.copy2(os.path.join(CSRC, f), os.path.join(out, "src", f))
    for f in sorted(os.listdir(INCLUDE)):
        shutil.copy2(os.path.join(INCLUDE, f), os.path.join(out, "src", f))
    shutil.copy2(os.path.join(HERE, "configure"), os.path.join(out, "configure"))
    os.chmod(os.path.join(out, "configure"), 0o755)
    shutil.copy2(os.path.join(HERE, "Makevars.in"), os.path.join(out, "src", "Makevars.in"))
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="checkout of the AccRQA reference")
    ap.add_argument("--out", required=True, help="package directory to write")
    a = ap.parse_args(argv)
    print(assemble(a.reference, a.out))


if __name__ == "__main__":
    main()
