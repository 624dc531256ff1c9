"""Build recipe for the oracle (test infrastructure only).

* ``oracle/liboracle.so``: the FP64 CPU restatement of the reference's VBD/XPBD path.
* ``oracle/_ref/libref_coloring.so``: the reference's own ``graphColoring.cpp`` compiled
  from the reference checkout, when that checkout is present. It is the only part of the
  reference that builds without its (absent) Eigen and TinyAD dependencies.

Both are git-ignored build products; the GPU host rebuilds the oracle from source.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def reference_root() -> str:
    """The reference checkout: $SPG_REFERENCE_ROOT, else a directory named `reference` beside
    this repository's root. When it is absent the reference's colouring is not built (the GPU
    hosts have no checkout; the tests that need it skip)."""
    env = os.environ.get("SPG_REFERENCE_ROOT")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp"]


def oracle_lib_path() -> str:
    return os.path.join(HERE, "liboracle.so")


def ref_lib_path() -> str:
    return os.path.join(HERE, "_ref", "libref_coloring.so")


def _needs(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def oracle_command() -> tuple[list[str], str, list[str]]:
    srcs = [os.path.join(HERE, "oracle.cpp")]
    deps = srcs + [os.path.join(HERE, "ad.h"), os.path.join(HERE, "energies.h")]
    out = oracle_lib_path()
    return ["g++", *CXXFLAGS, *srcs, "-o", out], out, deps


def ref_command() -> tuple[list[str], str, list[str]] | None:
    root = reference_root()
    src = os.path.join(root, "spg", "source", "utils", "graphColoring.cpp")
    inc = os.path.join(root, "spg", "include")
    if not os.path.exists(src):
        return None
    shim = os.path.join(HERE, "ref_coloring_shim.cpp")
    out = ref_lib_path()
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-I{inc}", src, shim, "-o", out]
    return cmd, out, [src, shim]


def commands(force: bool = False) -> list[list[str]]:
    cmds = []
    c, out, deps = oracle_command()
    if force or _needs(out, deps):
        cmds.append(c)
    r = ref_command()
    if r is not None:
        c, out, deps = r
        os.makedirs(os.path.dirname(out), exist_ok=True)
        if force or _needs(out, deps):
            cmds.append(c)
    return cmds


def build(force: bool = False) -> None:
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in commands(force)]
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
            raise RuntimeError(f"oracle build failed: {' '.join(c)}")


if __name__ == "__main__":
    build(force="--force" in sys.argv)
