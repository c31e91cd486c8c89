"""Build libops_fft.so in-tree (CUDA kernels for sm_103a + C++ API layer).

    python ops-fft_gb300/build.py [--jobs N] [--force]

Translation units are compiled in parallel with nvcc/g++ into ``_build/``
and linked into ``ops-fft_gb300/libops_fft.so`` (CUDA runtime linked
statically, only the ``aclfft*`` C API exported).  Objects are rebuilt when a
source or header is newer than them or the flags change.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libops_fft.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _sources():
    cu = sorted(glob.glob(os.path.join(HERE, "csrc", "*.cu")))
    cpp = sorted(glob.glob(os.path.join(HERE, "lib", "*.cpp")))
    return cu, cpp


def _headers():
    hs = []
    for pat in ("csrc/*.cuh", "csrc/*.h", "lib/*.h"):
        hs += glob.glob(os.path.join(HERE, pat))
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    return hs


def _flags_digest(flags):
    return hashlib.sha1(" ".join(flags).encode()).hexdigest()[:12]


def _compile(cmd, src, obj, stamp, newest_header, force):
    if not force and os.path.exists(obj) and os.path.exists(stamp):
        t = os.path.getmtime(obj)
        if t >= os.path.getmtime(src) and t >= newest_header:
            return obj, "cached"
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    open(stamp, "w").close()
    return obj, "built"


def build(jobs: int | None = None, force: bool = False, verbose: bool = False) -> str:
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include"), "-I", os.path.join(HERE, "csrc"), "-I", os.path.join(HERE, "lib")]
    cu_flags = ["-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
                "--expt-relaxed-constexpr", *inc]
    cxx = os.environ.get("CXX", "g++")
    cpp_flags = ["-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-Wall", "-Wno-unused-parameter",
                 "-I", os.path.join(cuda, "include"), *inc]
    digest = _flags_digest(cu_flags + cpp_flags)
    newest = max([os.path.getmtime(h) for h in _headers()] + [0.0])
    cu, cpp = _sources()
    jobs_list = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        jobs_list.append(([nvcc, *cu_flags, "-c", src, "-o", obj], src, obj, obj + "." + digest))
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        jobs_list.append(([cxx, *cpp_flags, "-c", src, "-o", obj], src, obj, obj + "." + digest))
    jobs = jobs or min(len(jobs_list), os.cpu_count() or 4)
    objs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, c, s, o, st, newest, force) for c, s, o, st in jobs_list]
        for f in futs:
            o, what = f.result()
            objs.append(o)
            if verbose:
                print(f"{what}: {os.path.basename(o)}")
    link = [nvcc, "-shared", *ARCH, "-o", LIB + ".tmp", *objs, "-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(link)}\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    args = ap.parse_args()
    path = build(args.jobs, args.force, verbose=True)
    print(path)


if __name__ == "__main__":
    sys.exit(main())
