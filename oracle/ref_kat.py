"""Builds oracle/_ref/ref_kat from the reference's own headers (read in place under the reference
tree, never copied) and writes tests/golden/smoothing_kernels.jsonl.

Run where the reference tree exists:  python oracle/ref_kat.py [reference_root]
(default: oracle/ref_root.py's lookup).
The output is committed; the GPU machine only reads the fixture.
"""
import os
import subprocess
import sys

try:
    from oracle.ref_root import require_reference_root
except ImportError:  # run as a script from oracle/
    from ref_root import require_reference_root

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_ref")
FIXTURE = os.path.join(REPO, "tests", "golden", "smoothing_kernels.jsonl")


def build(ref_root: str | None = None) -> str:
    ref_root = require_reference_root(ref_root)
    os.makedirs(OUT_DIR, exist_ok=True)
    exe = os.path.join(OUT_DIR, "ref_kat")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off",
           "-I", os.path.join(HERE, "ref_shim"), "-I", os.path.join(ref_root, "include"),
           os.path.join(HERE, "ref_kat.cpp"), "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def main(ref_root: str | None = None) -> None:
    exe = build(ref_root)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    os.makedirs(os.path.dirname(FIXTURE), exist_ok=True)
    with open(FIXTURE, "w") as f:
        f.write(out)
    print("wrote", FIXTURE, len(out.splitlines()), "lines")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
