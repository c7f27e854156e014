"""In-tree build of libgbint.so for sm_103a (nvcc, parallel translation units, no cmake).

Output: diffrg_gb300/lib/libgbint.so (git-ignored).  Every translation unit is compiled with
``-gencode arch=compute_103a,code=sm_103a -lineinfo``; host code is portable C++17 so that the
same sources build on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgbint.so")

SOURCES = ["engine.cu", "kernels_generic.cu", "kernels_fp32c.cu", "host_quadrature.cc", "serve.cc", "dloop.cu", "noalloc.cu",
           "slots.cu", "autotune.cc", "trace.cc"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-pthread", "-I", INCLUDE, "-I", CSRC,
            "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"] + ARCH


def _hash_inputs() -> str:
    h = hashlib.sha256()
    for d in (CSRC, os.path.join(INCLUDE), os.path.join(INCLUDE, "gbint"), os.path.join(INCLUDE, "gbint", "device")):
        if not os.path.isdir(d):
            continue
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p):
                h.update(f.encode())
                h.update(open(p, "rb").read())
    h.update(" ".join(_flags()).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    stamp = os.path.join(OBJ_DIR, "stamp")
    digest = _hash_inputs()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == digest:
        return LIB
    nv = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OBJ_DIR, src + ".o")
        lang = ["-x", "cu"]  # host-only .cc files include device headers too
        cmd = [nv] + _flags() + lang + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    cmd = [nv, "-shared"] + ARCH + ["-o", LIB] + objs + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
