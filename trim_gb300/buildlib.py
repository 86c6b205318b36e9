"""Build the trim_gb300 shared library in-tree (trim_gb300/_lib/).

CUDA sources are compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a); host C++ with g++.  No CMake.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libtrim_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INC = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(CUDA, "include")]


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "**", "*.cu"), recursive=True))
    cpp = sorted(glob.glob(os.path.join(CSRC, "**", "*.cpp"), recursive=True))
    return cu, cpp


def _headers_digest():
    h = hashlib.sha256()
    for p in sorted(glob.glob(os.path.join(CSRC, "**", "*.h*"), recursive=True) +
                    glob.glob(os.path.join(CSRC, "**", "*.cuh"), recursive=True) +
                    glob.glob(os.path.join(ROOT, "include", "**", "*.h*"), recursive=True)):
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def _obj(src, digest):
    rel = os.path.relpath(src, CSRC).replace(os.sep, "_")
    with open(src, "rb") as f:
        d = hashlib.sha256(f.read() + digest.encode()).hexdigest()[:12]
    return os.path.join(OUT, "obj", f"{rel}.{d}.o")


def _compile(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + p.stdout + p.stderr)
    return p.stderr


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    digest = _headers_digest()
    cu, cpp = _sources()
    jobs_ = []
    objs = []
    for s in cu:
        o = _obj(s, digest)
        objs.append(o)
        if not os.path.exists(o):
            jobs_.append([NVCC, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                          "--expt-relaxed-constexpr", *INC, "-c", s, "-o", o])
    for s in cpp:
        o = _obj(s, digest)
        objs.append(o)
        if not os.path.exists(o):
            jobs_.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function", *INC, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        for err in ex.map(_compile, jobs_):
            if verbose and err:
                sys.stderr.write(err)
    libdir = os.path.join(CUDA, "lib64")
    if not os.path.isdir(libdir):
        libdir = os.path.join(CUDA, "lib")
    tmp = LIB + ".tmp"
    link = ["g++", "-shared", "-o", tmp, *objs, "-L" + libdir, "-lcudart", "-lcusolver",
            "-Wl,-rpath," + libdir]
    _compile(link)
    os.replace(tmp, LIB)
    # stale objects from older sources
    keep = set(objs)
    for o in glob.glob(os.path.join(OUT, "obj", "*.o")):
        if o not in keep:
            os.remove(o)
    return LIB


def clean() -> None:
    shutil.rmtree(OUT, ignore_errors=True)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
