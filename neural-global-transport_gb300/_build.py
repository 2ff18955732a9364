"""In-tree build of ``libngt_ops.so`` for sm_103a.

Each ``csrc/*.cu`` file is compiled by nvcc in parallel into an object, then
the objects are linked into a shared library next to this file.  The CUDA
runtime is linked statically, so the library needs only the driver.
Rebuilds are skipped when no source or header is newer than the library.
ptxas's resource report of every kernel (registers, spills, shared memory) is
kept beside each object as ``_build/<source>.ptxas.txt``.
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libngt_ops.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xptxas", "-warn-spills", "-Xptxas", "-v", "-I", INCLUDE, "-I", CSRC]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = os.path.join(home, "bin", "nvcc")
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found (set CUDA_HOME)")
    return exe


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")) + [__file__]


def resource_report(src):
    """Path of ptxas's resource report for source ``src`` (written by the build)."""
    return os.path.join(BUILD, os.path.basename(src) + ".ptxas.txt")


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build_library(force=False, verbose=False, extra_flags=()):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [exe] + ARCH + FLAGS + list(extra_flags) + ["-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, res.stderr[-8000:]))
        with open(resource_report(src), "w") as f:
            f.write(res.stderr)
        if verbose:
            warnings = [l for l in res.stderr.splitlines() if "ptxas info" not in l]
            if warnings:
                print("\n".join(warnings))
        return obj

    srcs = _sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    cmd = [exe] + ARCH + ["-shared", "-o", tmp] + objs
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("link failed:\n%s" % res.stderr[-8000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build_library(force="--force" in sys.argv, verbose=True))
