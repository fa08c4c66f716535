"""TEST INFRASTRUCTURE ONLY.  Where the reference source tree is, for the recipes that compile
parts of it (oracle/ref_gpu.py, oracle/ref_kat.py).

The tree is taken from the environment variable AKUA_REFERENCE_ROOT, else from a directory named
`reference` beside this repository's own directory.  None when neither holds the reference's
include/AkuaEngine headers (the GPU machine has no reference tree; it uses what was built here).
"""
import os

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def reference_root():
    for cand in (os.environ.get("AKUA_REFERENCE_ROOT"),
                 os.path.join(os.path.dirname(REPO), "reference")):
        if cand and os.path.isdir(os.path.join(cand, "include", "AkuaEngine")):
            return cand
    return None


def require_reference_root(arg=None):
    root = arg or reference_root()
    if not root:
        raise RuntimeError("reference tree not found: set AKUA_REFERENCE_ROOT or pass its path")
    return root
