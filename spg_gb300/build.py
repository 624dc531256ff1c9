"""Build recipe of the shipped library ``spg_gb300/libspgx.so`` (sm_103a only).

Every translation unit is compiled in parallel with nvcc (``-gencode
arch=compute_103a,code=sm_103a``) and linked into one shared library that exports the C ABI
declared in ``include/spgx.h``. The library is built in-tree and git-ignored.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libspgx.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-lineinfo",
          f"-I{os.path.join(ROOT, 'include')}", f"-I{CSRC}", f"-I{os.path.join(HOST, 'include')}"]


# Extra flags per translation unit: the setup-time precomputations follow the host's FP64
# arithmetic operation by operation, so they are compiled without FMA contraction.
EXTRA = {"precompute.cu": ["--fmad=false"]}


def sources() -> list[str]:
    out = []
    for d in (CSRC, os.path.join(HOST, "src")):
        if not os.path.isdir(d):
            continue
        for f in sorted(os.listdir(d)):
            if f.endswith((".cu", ".cpp")):
                out.append(os.path.join(d, f))
    return out


def headers() -> list[str]:
    out = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    for d in (CSRC, os.path.join(HOST, "include")):
        for dirpath, _, files in os.walk(d):
            out += [os.path.join(dirpath, f) for f in files if f.endswith((".h", ".cuh"))]
    return [h for h in out if os.path.isfile(h)]


def _obj(src: str) -> str:
    rel = os.path.relpath(src, PKG).replace(os.sep, "_")
    return os.path.join(BUILD, rel + ".o")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if p.returncode != 0:
        sys.stderr.write(p.stdout.decode(errors="replace"))
        raise RuntimeError("build step failed: " + " ".join(cmd))


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = headers()
    srcs = sources()
    jobs = []
    for s in srcs:
        o = _obj(s)
        if force or _stale(o, [s] + hdrs):
            extra = (["-x", "cu"] if s.endswith(".cu") else []) + EXTRA.get(os.path.basename(s), [])
            jobs.append([NVCC, *ARCH, *COMMON, *extra, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    objs = [_obj(s) for s in srcs]
    if force or jobs or _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
