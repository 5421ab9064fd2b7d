"""Builds the replace::Replace facade test driver (TEST INFRASTRUCTURE).

The facade sources (replace_gb300/facade/*.cpp, include/replace/Replace.h)
are compiled against the in-memory OpenDB stand-in of oracle/refbuild and
linked with libgpl_gb300.so into replace_gb300/_build/facade_driver.  In
OpenROAD the same sources compile against the real OpenDB headers instead.
"""

from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
FACADE = os.path.join(ROOT, "replace_gb300", "facade")
OUT = os.path.join(ROOT, "replace_gb300", "_build")
DRIVER = os.path.join(OUT, "facade_driver")


def build(force: bool = False) -> str:
    from replace_gb300 import build as B
    lib = B.build()
    srcs = sorted(glob.glob(os.path.join(FACADE, "*.cpp"))) + [os.path.join(HERE, "facade_driver.cpp")]
    deps = srcs + glob.glob(os.path.join(FACADE, "*.h")) + [
        os.path.join(ROOT, "include", "gpl.h"), os.path.join(ROOT, "include", "replace", "Replace.h"),
        os.path.join(ROOT, "oracle", "refbuild", "opendb", "db.h"),
        os.path.join(ROOT, "oracle", "refbuild", "refnet_db.h"), lib]
    if not force and os.path.exists(DRIVER) and \
            os.path.getmtime(DRIVER) >= max(os.path.getmtime(d) for d in deps):
        return DRIVER
    tmp = DRIVER + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wno-unused-function",
           "-I", os.path.join(ROOT, "include"), "-I", FACADE,
           "-I", os.path.join(ROOT, "oracle", "refbuild"),
           "-o", tmp] + srcs + [lib, "-Wl,-rpath," + OUT, "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("facade driver build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(force=True))
