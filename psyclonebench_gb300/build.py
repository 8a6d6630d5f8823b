"""Builds libnl2d_gpu.so in-tree with nvcc for sm_103a (no torch extension
machinery: the library is a plain C-ABI shared object).

Every translation unit is compiled with -fmad=false: the FP64 step must
perform exactly the IEEE operations the reference's C source writes, with no
contracted multiply-adds, to be bit-identical to the reference.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT_DIR, "libnl2d_gpu.so")
# The reference executable's driver around the library (host C++ only).
DRIVER_SRC = "nl2d_driver_main.cpp"
DRIVER = os.path.join(OUT_DIR, "nemolite2d_gb300")
REPO = os.path.dirname(PKG)

SOURCES = [
    "nl2d_perkernel.cu",
    "nl2d_fused.cu",
    "nl2d_checksum.cu",
    "nl2d_capi.cu",
    "nl2d_mixed.cu",
    "nl2d_ensemble.cu",
    "nl2d_emu.cu",
    "nl2d_io.cpp",
    "tra_adv.cu",
    "nl2d_rates.cu",
    "nl2d_df.cu",
]
# The mixed-precision form has no bit-exactness contract: FMA contraction on.
PER_FILE_FLAGS = {"nl2d_mixed.cu": ["-fmad=true"]}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    "-Xcompiler", "-ffp-contract=off",
    "-I" + os.path.join(REPO, "include"),
]


def nvcc():
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if os.path.exists(cand) else "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
          if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(REPO, "include", "nl2d_gpu.h"))
    return hs


def build(force=False, verbose=False):
    """Compile (in parallel) and link the library; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    hdrs = _headers()
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            flags = [f for f in NVCC_FLAGS
                     if not (src in PER_FILE_FLAGS and f.startswith("-fmad"))]
            jobs.append([nvcc()] + flags + PER_FILE_FLAGS.get(src, []) + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for _ in ex.map(run, jobs):
            pass
    if force or jobs or _stale(LIB, objs):
        run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    drv_src = os.path.join(CSRC, DRIVER_SRC)
    if force or _stale(DRIVER, [drv_src, LIB] + hdrs):
        run([os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-ffp-contract=off",
             "-I" + os.path.join(REPO, "include"), drv_src, "-o", DRIVER, "-L" + OUT_DIR,
             "-lnl2d_gpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
