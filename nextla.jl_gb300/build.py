"""Build the in-tree C-ABI library ``libnextla_gb300.so`` for sm_103a.

Every ``csrc/*.cu`` translation unit is compiled by nvcc in parallel, then
linked into one shared library next to this file.  The CUDA runtime is linked
statically; the driver API (tensor-map encoding) is reached through
``cudaGetDriverEntryPoint``, so the library has no link-time dependency on
``libcuda.so`` and cross-compiles on a machine without a GPU.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libnextla_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) +
                  glob.glob(os.path.join(HERE, "..", "include", "*.h")))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library if any source is newer than it."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = _sources()
    hdrs = _headers()
    objs = [os.path.join(OBJ_DIR, os.path.basename(s)[:-3] + ".o") for s in srcs]
    cc = nvcc()
    flags = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
             "--expt-relaxed-constexpr"] + ARCH

    def compile_one(pair):
        src, obj = pair
        if not force and not _stale(obj, [src] + hdrs):
            return obj
        tmp = obj + ".tmp%d.o" % os.getpid()
        cmd = [cc] + flags + ["-c", src, "-o", tmp]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (os.path.basename(src), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        os.replace(tmp, obj)
        return obj

    workers = max(1, min(len(srcs), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))

    if force or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        cmd = [cc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
