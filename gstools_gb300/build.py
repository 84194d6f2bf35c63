"""Build the gstools_gb300 CUDA library in-tree with nvcc for sm_103a.

``python -m gstools_gb300.build`` (or ``build()``) compiles every translation
unit under ``csrc/`` in parallel and links ``libgstools_gb300.so`` next to
this file.  The library exposes the C ABI declared in
``include/gstools_gb300.h`` and links the CUDA runtime statically, so the only
runtime dependency is the NVIDIA driver.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(PKG_DIR)
CSRC_DIR = os.path.join(PKG_DIR, "csrc")
INCLUDE_DIR = os.path.join(ROOT_DIR, "include")
BUILD_DIR = os.path.join(ROOT_DIR, "_build", "gstools_gb300")
LIB_NAME = "libgstools_gb300.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
# cuBLAS runs the plain FP16 slice GEMMs of the FP64 kriging variance
LINK_LIBS = ["-lcublas"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler", "-fPIC",
    "-Xcompiler", "-O2",
    "--expt-relaxed-constexpr",
]


def nvcc_path():
    """Locate nvcc (CUDA_HOME, PATH, then /usr/local/cuda)."""
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.exists(os.path.join(home, "bin", "nvcc")):
        return os.path.join(home, "bin", "nvcc")
    found = shutil.which("nvcc")
    if found:
        return found
    default = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(default):
        return default
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def sources():
    return sorted(
        os.path.join(CSRC_DIR, f)
        for f in os.listdir(CSRC_DIR)
        if f.endswith(".cu")
    )


def _headers_mtime():
    paths = [os.path.join(CSRC_DIR, f) for f in os.listdir(CSRC_DIR)
             if f.endswith((".cuh", ".h"))]
    paths += [os.path.join(INCLUDE_DIR, f) for f in os.listdir(INCLUDE_DIR)]
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src, extra, verbose):
    obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc_path(), *ARCH_FLAGS, *NVCC_FLAGS, *extra,
           "-I", INCLUDE_DIR, "-I", CSRC_DIR, "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(
            f"nvcc failed for {os.path.basename(src)}:\n{proc.stdout}\n"
            f"{proc.stderr}"
        )
    return obj, proc.stdout + proc.stderr


def up_to_date():
    """Whether the library is newer than every source and header."""
    if not os.path.exists(LIB_PATH):
        return False
    newest = max([os.path.getmtime(s) for s in sources()] + [_headers_mtime()])
    return os.path.getmtime(LIB_PATH) >= newest


def build(force=False, verbose=False, ptxas_info=False, jobs=None):
    """Compile and link the library; returns its path."""
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(jobs) as pool:
        results = list(pool.map(lambda s: _compile(s, extra, verbose), srcs))
    if ptxas_info:
        for _, log in results:
            sys.stdout.write(log)
    objs = [o for o, _ in results]
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc_path(), *ARCH_FLAGS, "-shared", "-o", tmp, *objs, *LINK_LIBS]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"link failed:\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                 ptxas_info="--ptxas-info" in sys.argv)
    print(path)
