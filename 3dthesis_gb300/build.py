"""Builds the native parts in-tree with nvcc (no cmake, no setuptools).

Products (git-ignored, rebuilt on every machine):
  3dthesis_gb300/libthesis_gb300.so   the C-ABI library (CUDA sm_103a + host C++)
  3dthesis_gb300/thesis_gb300         the command-line driver (``thesis_gb300 ParamInput.txt``)
  oracle/liboracle.so                 the CPU oracle (test infrastructure only)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libthesis_gb300.so")
CLI = os.path.join(PKG, "thesis_gb300")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def nvcc() -> str:
    p = os.path.join(CUDA_HOME, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _flags() -> list:
    # host code: no FMA contraction, so the deck arithmetic rounds as the reference's does
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC] + ARCH


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "thesis_gb300.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + _flags() + ["-c", src, "-o", obj]
    if verbose and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build_library(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")) and f != "thesis_cli.cpp")
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        subprocess.run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs, check=True)
    cli_src = os.path.join(CSRC, "thesis_cli.cpp")
    if os.path.exists(cli_src):
        cli_obj = _compile(cli_src, False)
        if not os.path.exists(CLI) or os.path.getmtime(cli_obj) > os.path.getmtime(CLI) \
                or os.path.getmtime(LIB) > os.path.getmtime(CLI):
            subprocess.run([nvcc()] + ARCH + ["-o", CLI, cli_obj, "-L" + PKG, "-lthesis_gb300",
                            "-Xlinker", "-rpath,$ORIGIN"], check=True)
    return LIB


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return os.path.join(ROOT, "oracle", "liboracle.so")


if __name__ == "__main__":
    build_library(verbose="-v" in sys.argv)
    build_oracle()
    print(LIB)
