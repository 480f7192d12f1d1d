"""Builds libcrngpu.so (the C-ABI library) in-tree for sm_103a with nvcc.

Translation units are compiled in parallel; dxt_encode.cu and hc_encode.cu are compiled with
--fmad=false because their float/double code must round exactly like the reference's (no
contraction): the tile errors of the clustered path decide its tile layouts.
Usage: python -m crunch2_gb300.build   (or crunch2_gb300.build.build())
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcrngpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
               "-Xcompiler", "-ffp-contract=off"]

UNITS = [
    ("crn_file.cpp", []),
    ("crn_pack.cpp", []),
    ("capi.cpp", []),
    ("crn_transcode.cu", []),
    ("encode_api.cu", []),
    ("encode_batch.cu", []),
    ("dxt_encode.cu", ["--fmad=false"]),
    ("mlp.cu", []),
    ("hc_encode.cu", ["--fmad=false"]),
    ("mip_gen.cu", ["--fmad=false"]),
    ("crnlib_compat.cpp", []),
]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcrngpu.so")


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith(".h")]
    for h in ("crngpu.h", "crnlib_compat.h"):
        deps.append(os.path.join(os.path.dirname(HERE), "include", h))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nv = nvcc()
    procs, objs = [], []
    for name, extra in UNITS:
        src = os.path.join(SRC, name)
        obj = os.path.join(OUT_DIR, name + ".o")
        objs.append(obj)
        if not _stale(obj, src):
            continue
        cmd = [nv, *ARCH, *NVCC_COMMON, *extra, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for name, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((name, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(f"--- {n}\n{o}" for n, o in failed)
        raise RuntimeError("libcrngpu build failed:\n" + msg)
    if procs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nv, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("libcrngpu link failed:\n" + r.stdout.decode(errors="replace"))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
