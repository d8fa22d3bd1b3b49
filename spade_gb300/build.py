"""In-tree build of libgbns.so (the CUDA library) for sm_103a.

Compiles every translation unit under spade_gb300/csrc in parallel with
nvcc (one -gencode for sm_103a; every TU is a self-contained device module) and links them into
spade_gb300/_build/libgbns.so.  Rebuilds only when a source is newer than the
library.
"""
import concurrent.futures
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgbns.so")
INCLUDE = os.path.join(ROOT, "include")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17",
                "-Xcompiler", "-fPIC,-ffp-contract=off",
                "-diag-suppress", "177",
                "-I" + INCLUDE, "-I" + CSRC]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _deps())


# Translation units whose FP64 arithmetic must round exactly like the
# reference's CPU code: no fused multiply-add contraction.
NO_FMA = ("flux_f64x_", "state.cu", "batch_flux_f64x", "source.cu", "bflux_", "exchange.cu")


def _compile(src):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    extra = ["-fmad=false"] if any(k in os.path.basename(src) for k in NO_FMA) else []
    cmd = [NVCC] + FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-4000:]))
    return obj


def build(force=False, verbose=False):
    """Builds libgbns.so if needed and returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    workers = max(1, min(len(srcs), os.cpu_count() or 4))
    with concurrent.futures.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-Xcompiler", "-fPIC"] + objs + ["-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
