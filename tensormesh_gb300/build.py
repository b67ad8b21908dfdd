"""In-tree build of the C-ABI shared library ``_lib/libtmgb300.so``.

Every ``csrc/*.cu`` file is compiled for sm_103a only (one -gencode) in
parallel with nvcc, then linked with ``-shared``.  Rebuilds are incremental
(object newer than its source and every header).  The build runs on the
machine that will load the library; nothing compiled on another
architecture is reused.
"""
from __future__ import annotations

import glob
import os
import platform
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_NAME = "libtmgb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tensormesh_gb300")


def lib_path() -> str:
    return os.path.join(OUT_DIR, platform.machine(), LIB_NAME)


def _newest_header() -> float:
    hdrs = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(h) for h in hdrs), default=0.0)


def build(verbose: bool = False, jobs: int | None = None, extra_flags=()) -> str:
    """Compile and link the library; returns its path."""
    nvcc = nvcc_path()
    out_dir = os.path.dirname(lib_path())
    obj_dir = os.path.join(out_dir, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr_time = _newest_header()
    objs, todo = [], []
    for src in sources:
        obj = os.path.join(obj_dir, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            todo.append((src, obj))

    def compile_one(job):
        src, obj = job
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra_flags, "-I", INCLUDE, "-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{res.stderr}")
        return res.stderr

    if todo:
        with ThreadPoolExecutor(jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for msg in ex.map(compile_one, todo):
                if verbose and msg.strip():
                    print(msg)
    lib = lib_path()
    if todo or not os.path.exists(lib):
        cmd = [nvcc, *ARCH, "-shared", "-o", lib, *objs, "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr}")
    return lib


if __name__ == "__main__":
    print(build(verbose=True))
