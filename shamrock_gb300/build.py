"""Build libgbsph.so (the C-ABI library) in-tree with nvcc for sm_103a.

Translation units are compiled in parallel.  Files whose FP64 arithmetic must match
the reference evaluation order bit for bit are compiled with fused multiply-add
disabled; the mixed-precision file keeps FMA on.

    python -m shamrock_gb300.build          # build if sources are newer
    python -m shamrock_gb300.build --force  # rebuild everything
Environment: GBSPH_PTXAS_VERBOSE=1 adds -Xptxas -v (register/spill report).
"""

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbsph.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                 "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]
# FP64 units whose results are compared bit for bit with the oracle
EXACT = {"tree.cu", "neigh.cu", "ghosts.cu", "sph64.cu", "scan.cu", "driver.cu"}
# FP32-mixed pair kernels: approximate FP32 division / square root, denormals flushed
FAST32 = {"sph_mixed.cu", "sph_comp.cu"}


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libgbsph.so")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "gbsph.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def _compile(src):
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    flags = list(COMMON)
    flags += ["-fmad=false"] if src in EXACT else ["-fmad=true"]
    if src in FAST32:
        flags += ["-prec-div=false", "-prec-sqrt=false", "-ftz=true"]
    if os.environ.get("GBSPH_PTXAS_VERBOSE"):
        flags += ["-Xptxas", "-v"]
    cmd = [nvcc()] + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    return src, r.returncode, r.stdout + r.stderr, obj


def build(force=False, verbose=False):
    """Compile every .cu under csrc/ and link libgbsph.so; returns the library path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    objs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        for src, rc, out, obj in ex.map(_compile, srcs):
            if verbose or os.environ.get("GBSPH_PTXAS_VERBOSE"):
                sys.stderr.write(out)
            if rc != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{out}")
            objs.append(obj)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
