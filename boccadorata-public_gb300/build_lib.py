"""Builds the in-tree CUDA library libbd_gb300.so for sm_103a (nvcc, no cmake).

Run as ``python build_lib.py`` or through ``__graft_entry__.build()``.  Each
translation unit is compiled in parallel; the objects are linked into one shared
library next to this file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libbd_gb300.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["bd_api.cu", "k_sigma2.cu", "k_lanczos.cu", "k_dyson.cu", "k_eig.cu", "k_sort.cu", "bd_files.cu",
           "k_coupling_tc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                    "-I", os.path.join(HERE, "..", "include")]
    if ptxas_info:
        flags += ["-Xptxas", "-v"]

    def one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc()] + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        res = list(ex.map(one, SOURCES))
    if verbose or ptxas_info:
        for _, err in res:
            sys.stderr.write(err)
    objs = [o for o, _ in res]
    tmp = OUT + ".tmp"
    r = subprocess.run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
