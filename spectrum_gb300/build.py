"""Build recipe of the CUDA library: every translation unit of csrc/ compiled in parallel with
nvcc for sm_103a, linked into spectrum_gb300/_lib/libspx.so (in-tree, git-ignored).

Run as ``python -m spectrum_gb300.build`` or through ``__graft_entry__.build()``. A unit is
recompiled only when it or a header is newer than its object file.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, os.environ.get("SPX_LIB_DIR", "_lib"))
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libspx.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build spectrum_gb300")


def sources() -> list[str]:
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cc")))


def _newest_header() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hh", ".cuh"))]
    hs.append(os.path.join(os.path.dirname(PKG), "include", "spx.h"))
    return max(os.path.getmtime(h) for h in hs if os.path.exists(h))


def _compile(src: str, nvcc: str, extra: list[str]) -> tuple[str, int, str]:
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    # The FP32 kernels use the hardware approximations of division, square root, log, exp, sin,
    # cos and pow (relative errors of a few 1e-7). The FP64 kernels keep IEEE arithmetic and are
    # compiled without multiply-add contraction, so every +, -, *, / and sqrt rounds as in the
    # reference's own (uncontracted) build and in the oracle.
    if "_f32" in src:  # spx_k_<family>_f32.cu and the FP32 units specialised for one diffusion class
        fast = ["-use_fast_math"]
    elif src.endswith(("_f64.cu", "_f64fd.cu", "_f64rk.cu", "_f64fdrk.cu")):
        fast = ["-fmad=false"]
    else:
        fast = []
    cmd = [nvcc, *lang, *ARCH, *CFLAGS, *fast, *extra, "-c", path, "-o", obj]
    # an object is reused only if it is newer than its sources and was made by the same command
    stamp = obj + ".cmd"
    line = " ".join(cmd)
    if (os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == line
            and os.path.getmtime(obj) >= max(os.path.getmtime(path), _newest_header())):
        return obj, 0, ""
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode == 0:
        with open(stamp, "w") as f:
            f.write(line)
    return obj, r.returncode, r.stdout + r.stderr


def build(verbose: bool = False, extra: list[str] | None = None, jobs: int | None = None) -> str:
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    extra = (extra or []) + os.environ.get("SPX_NVCC_FLAGS", "").split()
    srcs = sources()
    jobs = jobs or min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, nvcc, extra), srcs))
    for obj, rc, log in results:
        if rc != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(obj)}:\n{log}")
        if verbose and log:
            print(log)
    objs = [r[0] for r in results]
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
