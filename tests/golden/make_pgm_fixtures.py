"""Copies the reference's symmetric PGM power-flow fixtures into tests/golden/pgm.

The fixtures (input, update batch, expected node voltages) come from the
reference's tests/data/pgm/powerflow/symmetric/<case>/, which adopts them from
the Power Grid Model project (MPL-2.0; each case's README with its SPDX lines
is copied beside it).  Run from the repository root:

    python tests/golden/make_pgm_fixtures.py [reference checkout]
"""
import os
import shutil
import sys

CASES = ["basic-node", "node", "line", "shunt", "sym_load", "sym_gen", "source",
         "transmission-case", "transformer", "distribution-case", "three_winding_transformer"]
FILES = ["README.md", "input.json", "sym_output.json", "update_batch.json", "sym_output_batch.json"]


def main(ref: str) -> None:
    src_root = os.path.join(ref, "tests", "data", "pgm", "powerflow", "symmetric")
    dst_root = os.path.join(os.path.dirname(os.path.abspath(__file__)), "pgm")
    for case in CASES:
        os.makedirs(os.path.join(dst_root, case), exist_ok=True)
        for f in FILES:
            src = os.path.join(src_root, case, f)
            if os.path.exists(src):
                shutil.copyfile(src, os.path.join(dst_root, case, f))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["GRIDOXIDE_REFERENCE"])
