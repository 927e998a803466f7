"""Builds the native library of the BVE path in-tree.

``build()`` compiles every CUDA translation unit for sm_103a (GB300) with nvcc and the
host translation units with g++, in parallel, and links ``_build/liblpm_bve.so`` next
to this file.  Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liblpm_bve.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")

CU_SOURCES = ["pair_kernels.cu", "stage_kernels.cu", "probe.cu", "noalloc.cu", "norms.cu", "ic.cu", "octree.cu", "tree.cu"]
CXX_SOURCES = ["engine.cpp", "mesh.cpp", "server.cpp", "snapshot.cpp"]


def _nvcc() -> str:
    p = os.path.join(CUDA_HOME, "bin", "nvcc")
    return p if os.path.exists(p) else (shutil.which("nvcc") or "nvcc")


def _headers():
    hs = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".hpp", ".cuh")):
                hs.append(os.path.join(d, f))
    return hs


def _stale(obj: str, src: str, headers) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src, *headers, __file__])


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = _headers()
    incs = [f"-I{INCLUDE}", f"-I{CSRC}", f"-I{os.path.join(CUDA_HOME, 'include')}"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if _stale(o, s, headers):
            cmd = [_nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", "-diag-suppress", "177", *incs, "-c", s, "-o", o]
            jobs.append((src, cmd))
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if _stale(o, s, headers):
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall", *incs, "-c", s, "-o",
                   o]
            jobs.append((src, cmd))
    procs = [(src, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for src, cmd in jobs]
    errors = []
    for src, cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"--- {src}: {' '.join(cmd)}\n{out}")
        elif verbose and out.strip():
            print(out, file=sys.stderr)
    if errors:
        raise RuntimeError("native build failed:\n" + "\n".join(errors))
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", LIB, *objs,
               f"-L{os.path.join(CUDA_HOME, 'lib64')}", "-lcudart", "-lpthread"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    _build_examples(incs)
    return LIB


EXAMPLES = ["bve_solid_body", "bve_serve"]


def _build_examples(incs):
    """The C++ drop-in driver(s), linked against the library with an rpath to _build/."""
    for name in EXAMPLES:
        src = os.path.join(HERE, "examples", name + ".cpp")
        exe = os.path.join(OUT, name)
        deps = [src, LIB, *_headers()]
        if os.path.exists(exe) and all(os.path.getmtime(d) <= os.path.getmtime(exe) for d in deps):
            continue
        cmd = ["g++", "-O2", "-std=c++17", "-pthread", *incs, src, "-o", exe, f"-L{OUT}", "-llpm_bve",
               f"-L{os.path.join(CUDA_HOME, 'lib64')}", "-lcudart",
               f"-Wl,-rpath,{OUT}:{os.path.join(CUDA_HOME, 'lib64')}"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("example build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


if __name__ == "__main__":
    print(build(verbose=True))
