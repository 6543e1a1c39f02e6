"""Copies the reference's example inputs that tests/golden/ref_examples.json
was made from into tests/golden/_refdata/ (git-ignored), so that tests can
read them where the reference checkout is absent.

The files are the reference project's own example data (mammals and
Primates trees and family tables, an error-model file, a lambda tree, a
root-size distribution); they are inputs of the parity tests, not part of
the product, and are never committed. Run where the checkout exists
(CAFE_REFERENCE, or the default the oracle's recipe uses):
    python tests/golden/stage_examples.py
"""
from __future__ import annotations

import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_refdata")


def files():
    meta = json.load(open(os.path.join(HERE, "ref_examples.json")))
    out = set()
    for c in meta["cases"]:
        for k in ("tree", "families", "error", "lambda_tree", "rootdist"):
            if c.get(k):
                out.add(c[k])
    return sorted(out)


def stage(reference: str) -> int:
    n = 0
    for rel in files():
        src = os.path.join(reference, rel)
        dst = os.path.join(OUT, rel)
        if os.path.exists(dst) and os.path.getsize(dst) == os.path.getsize(src):
            continue
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(src, dst)
        n += 1
    return n


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    ref = oracle.reference_dir()
    if ref is None:
        raise SystemExit("no reference checkout (set CAFE_REFERENCE)")
    print(f"staged {stage(ref)} files into {OUT}")


if __name__ == "__main__":
    main()
