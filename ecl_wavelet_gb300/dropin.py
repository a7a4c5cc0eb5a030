"""Builds the C++ drop-in example (tests/cpp/dropin_example.cu) against
libewt.so, the way a user of the reference's header API would."""
import os
import subprocess

from . import buildlib

REPO = buildlib.REPO
SRC = os.path.join(REPO, "tests", "cpp", "dropin_example.cu")
BIN = os.path.join(REPO, "tests", "cpp", "bin", "dropin_example")


def build_example() -> str:
    lib = buildlib.build()
    deps = [SRC, lib] + buildlib.headers()
    if not buildlib._stale(BIN, deps):
        return BIN
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    cmd = ([buildlib.nvcc()] + buildlib.ARCH
           + ["-O2", "-std=c++20", "-I", buildlib.INCLUDE, SRC, "-o", BIN,
              "-L", buildlib.PKG, "-lewt", "-Xlinker",
              "-rpath=" + buildlib.PKG])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("drop-in example failed to build:\n%s\n%s" % (
            " ".join(cmd), r.stderr[-4000:]))
    return BIN
