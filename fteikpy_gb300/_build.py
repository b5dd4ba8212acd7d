"""Build the CUDA library ``_lib/libfteik_gb300.so`` in-tree with nvcc (sm_103a).

Every translation unit under ``csrc/`` is compiled in parallel, then linked into
one shared library that exports the C ABI declared in ``include/fteik_gb300.h``.
The library is compiled with ``--fmad=false``: the kernels reproduce the
reference's arithmetic operation by operation and must not be contracted.
"""

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "_lib")
LIB_NAME = "libfteik_gb300.so"
LIB_PATH = os.path.join(LIB_DIR, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "--fmad=false",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC,-O2",
    "-I" + INCLUDE,
    "-I" + CSRC,
]

# Everything that reproduces the reference's arithmetic is compiled without
# multiply-add contraction (bitwise parity). The adjoint's partials have no
# such contract, so that file may contract.
CONTRACTED = {"adjoint3d.cu"}


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the fteik_gb300 CUDA library cannot be built")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    files = sources()
    files += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    files.append(os.path.join(INCLUDE, "fteik_gb300.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False):
    """Compile the library if needed; return its path."""
    if not force and up_to_date():
        return LIB_PATH
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        flags = NVCC_FLAGS
        if os.path.basename(src) in CONTRACTED:
            flags = [f for f in flags if not f.startswith("--fmad")] + ["--fmad=true"]
        cmd = [nvcc] + flags + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
