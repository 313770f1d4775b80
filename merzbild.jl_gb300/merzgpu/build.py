"""Build libmerzgpu.so (the C-ABI CUDA library) in-tree for sm_103a.

Each translation unit in ../csrc is compiled by nvcc in parallel and linked
into merzgpu/lib/libmerzgpu.so.  Nothing is installed outside the package.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
OBJ = os.path.join(ROOT, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libmerzgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(s for s in glob.glob(os.path.join(CSRC, "*.cu")) if not os.path.basename(s).startswith("_"))


STAMP = os.path.join(LIBDIR, ".stamp")


def _stamp(extra_flags=()) -> str:
    """Digest of every input: source names, sizes, contents and flags."""
    h = hashlib.sha1()
    files = sorted(glob.glob(os.path.join(CSRC, "*"))) + [os.path.join(os.path.dirname(ROOT), "include", "merzgpu.h")]
    for f in files:
        if os.path.isfile(f):
            h.update(os.path.basename(f).encode())
            with open(f, "rb") as fh:
                h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS + list(extra_flags)).encode())
    return h.hexdigest()


def up_to_date(extra_flags=()) -> bool:
    if not (os.path.exists(LIB) and os.path.exists(STAMP)):
        return False
    with open(STAMP) as f:
        return f.read().strip() == _stamp(extra_flags)


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    if not force and up_to_date(extra_flags or ()):
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    exe = nvcc()
    flags = NVCC_FLAGS + list(extra_flags or [])
    srcs = _sources()

    def compile_one(src):
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
        cmd = [exe] + ARCH + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        return src, obj, r

    objs = []
    errors = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        for src, obj, r in ex.map(compile_one, srcs):
            if r.returncode != 0:
                errors.append(f"--- {os.path.basename(src)}\n{r.stdout}{r.stderr}")
            else:
                objs.append(obj)
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    r = subprocess.run([exe] + ARCH + ["-shared", "-o", tmp] + objs, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(_stamp(extra_flags or ()))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
