"""Build the host harness of the reference's own operator code (test infrastructure).

Each harness library is one translation unit streamed into ``g++`` on stdin:

1. a head that mirrors the include list of the reference's ``.cu.cc`` file
   (the reference headers are included from where they lie),
2. the reference's device functions and ``__global__`` kernel bodies, read
   from the reference's ``.cu.cc`` files by line range (``#line`` keeps
   diagnostics pointing at the reference file) -- the host launcher code in
   those files uses ``<<<...>>>`` and cannot be compiled as C++, so only the
   device-side ranges are taken,
3. a driver that restates the launchers' host loops and runs every kernel
   body once per emulated thread (``ref_prelude.h``).

Nothing from the reference is written to disk; the only outputs are the
shared libraries in ``oracle/_ref/``.  The reference tree must be present
(it is only in the development container, never on the GPU host), so this
runs where the golden vectors are generated.

Usage: ``python oracle/refharness/build.py [--ref /path/to/reference]`` (default: the
``NGT_REFERENCE_ROOT`` environment variable, else the development container's tree)
"""
import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
# where the reference tree lies in the development container (this recipe reads
# the reference's sources from there); NGT_REFERENCE_ROOT or --ref point elsewhere
DEFAULT_REF = os.environ.get("NGT_REFERENCE_ROOT", "/root/reference")
SRC = "phitest/render/cuda/src"

# (head, [(file, first_line, last_line)], driver, output)
UNITS = {
    "v2": ("head_v2.inc", [
        ("raymarch_grid.cu.cc", 86, 98),     # globalThreadIdx3D, isInDimensions
        ("raymarch_grid.cu.cc", 109, 252),   # ray/AABB setup and forward kernel
        ("raymarch_grid.cu.cc", 458, 521),   # gradient normalisation and gradient kernel
    ], "driver_v2.inc", "libref_v2.so"),
    "v1": ("head_v1.inc", [
        ("resample_grid.cu.cc", 255, 267),   # kSample3D
        ("resample_grid.cu.cc", 604, 623),   # kSampleGrid3DLuT
        ("resample_grid.cu.cc", 877, 1131),  # atomic helpers, quadratic and trilinear scatter
        ("resample_grid.cu.cc", 1133, 1151),  # kNormalize3DGradients
        ("resample_grid.cu.cc", 1160, 1190),  # kScatter3DGradients
        ("resample_grid.cu.cc", 1420, 1450),  # kScatterLuT3DGradients
        ("resample_grid.cu.cc", 1702, 1717),  # kComputeLoD3D
    ], "driver_v1.inc", "libref_v1.so"),
    "rb": ("head_rb.inc", [
        ("reduce_blend.cu.cc", 34, 80),      # kBlend, kBlendGrad
    ], "driver_rb.inc", "libref_rb.so"),
}


def compose(ref, unit):
    head, ranges, driver, _ = UNITS[unit]
    parts = [open(os.path.join(HERE, head)).read()]
    for fname, a, b in ranges:
        path = os.path.join(ref, SRC, fname)
        with open(path) as f:
            lines = f.read().split("\n")
        parts.append('#line %d "%s"\n' % (a, path))
        parts.append("\n".join(lines[a - 1:b]) + "\n")
    parts.append('#line 1 "%s"\n' % os.path.join(HERE, driver))
    parts.append(open(os.path.join(HERE, driver)).read())
    return "".join(parts)


def build(ref=DEFAULT_REF, units=("v1", "v2", "rb"), cxx="g++", verbose=False):
    os.makedirs(OUT, exist_ok=True)
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    outputs = []
    for u in units:
        out = os.path.join(OUT, UNITS[u][3])
        cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-w", "-x", "c++", "-",
               "-I", HERE, "-I", os.path.join(HERE, "shim"), "-I", os.path.join(ref, SRC),
               "-I", os.path.join(ref, "lib", "glm"), "-I", cuda_inc, "-o", out]
        res = subprocess.run(cmd, input=compose(ref, u), text=True, capture_output=True)
        if res.returncode != 0:
            sys.stderr.write(res.stderr[-6000:])
            raise RuntimeError("reference harness unit %s failed to compile" % u)
        if verbose:
            print("built", out)
        outputs.append(out)
    return outputs


def available(ref=DEFAULT_REF):
    return os.path.isdir(os.path.join(ref, SRC))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=DEFAULT_REF)
    ap.add_argument("units", nargs="*", default=["v1", "v2", "rb"])
    a = ap.parse_args()
    build(a.ref, a.units, verbose=True)
