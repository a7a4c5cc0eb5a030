"""Builds the C++ drop-in programs (tests/cpp/*.cu: the tree example and the
standalone BitArray / RankSelect example) against libewt.so, the way a user
of the reference's header API would."""
import os
import subprocess

from . import buildlib

REPO = buildlib.REPO
CPP = os.path.join(REPO, "tests", "cpp")


def build_example(name: str = "dropin_example") -> str:
    """Compiles tests/cpp/<name>.cu against libewt.so; returns the binary."""
    src = os.path.join(CPP, name + ".cu")
    binary = os.path.join(CPP, "bin", name)
    lib = buildlib.build()
    deps = [src, lib] + buildlib.headers()
    if not buildlib._stale(binary, deps):
        return binary
    os.makedirs(os.path.dirname(binary), exist_ok=True)
    cmd = ([buildlib.nvcc()] + buildlib.ARCH
           + ["-O2", "-std=c++20", "-I", buildlib.INCLUDE, src, "-o", binary,
              "-L", buildlib.PKG, "-lewt", "-Xlinker",
              "-rpath=" + buildlib.PKG])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("drop-in program failed to build:\n%s\n%s" % (
            " ".join(cmd), r.stderr[-4000:]))
    return binary
