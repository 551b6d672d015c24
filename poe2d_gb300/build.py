"""Build the native library ``libpoe2d.so`` (and the drop-in CLI) in-tree.

Compiles the CUDA kernels for sm_103a only and the C++ host library with
nvcc, one process per translation unit, into ``poe2d_gb300/_build/``.
``-fmad=false`` / ``-ffp-contract=off`` keep every a*b+c as two IEEE
operations, which is how the reference's arithmetic is specified.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpoe2d.so")
CLI = os.path.join(BUILD, "poe2d_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["poe2d_tile_fast.cu", "poe2d_tile_exact.cu", "poe2d_tile_exact_any.cu", "poe2d_tile_fast16.cu", "poe2d_tile.cu", "poe2d_api.cpp",
           "poe2d_setup.cpp", "sg_gemm.cu", "sg_ops.cu", "sg_net.cpp"]


def nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand) and shutil.which(cand) is None:
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build poe2d_gb300")
    return cand


def cuda_lib_dir():
    nv = os.path.realpath(nvcc())
    root = os.path.dirname(os.path.dirname(nv))
    for sub in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        d = os.path.join(root, sub)
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    return os.path.join(root, "lib64")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                   "-I", os.path.join(ROOT, "include")]


def resource_report(src):
    """ptxas's per-kernel resource lines (registers, stack, spills) of a .cu unit, kept by the build."""
    return os.path.join(BUILD, os.path.splitext(src)[0] + ".ptxas.txt")


def _compile(src):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + _flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd[cmd.index("-c")] = "-x"
        cmd.insert(cmd.index("-x") + 1, "c++")
        cmd.insert(cmd.index("c++") + 1, "-c")
    else:
        cmd[1:1] = ["-Xptxas", "-v"]   # reports only; code generation is unchanged
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), out.stdout, out.stderr))
    if src.endswith(".cu"):
        with open(resource_report(src), "w") as f:
            f.write(out.stderr)
    return obj


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile libpoe2d.so (and the CLI) if any source is newer than it."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "poe2d.h")]
    reports = [resource_report(s) for s in SOURCES if s.endswith(".cu")]
    if force or _stale(LIB, deps) or not all(os.path.exists(r) for r in reports):
        with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
            objs = list(ex.map(_compile, SOURCES))
        libdir = cuda_lib_dir()
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", LIB + ".tmp"] + objs + [
            "-Xlinker", "-rpath," + libdir, "-L", libdir]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), out.stdout, out.stderr))
        os.replace(LIB + ".tmp", LIB)
        if verbose:
            print("built", LIB)
    cli_src = os.path.join(CSRC, "poe2d_cli.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB])):
        cmd = [nvcc(), "-O2", "-std=c++17", "-x", "c++", cli_src, "-o", CLI, "-I", os.path.join(ROOT, "include"),
               "-L", BUILD, "-lpoe2d", "-Xlinker", "-rpath,$ORIGIN", "-Xlinker", "-rpath," + cuda_lib_dir(),
               "-cudart", "shared"]
        out = subprocess.run(cmd, capture_output=True, text=True)
        if out.returncode != 0:
            raise RuntimeError("CLI build failed: %s\n%s%s" % (" ".join(cmd), out.stdout, out.stderr))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
