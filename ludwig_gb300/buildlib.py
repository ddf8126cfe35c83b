"""Build libludwig_gb.so in-tree (nvcc for sm_103a + gcc for the C host side).

FP64 translation units are compiled with ``--fmad=false`` so that each
multiply and add rounds on its own, as in the reference's serial build;
the reduced-precision units keep fused multiply-add.
"""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libludwig_gb.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
CU_SOURCES = [
    ("lgb_ref64.cu", ["--fmad=false"]),
    ("lgb_fused64.cu", ["--fmad=false"]),
    ("lgb_stats.cu", ["--fmad=false"]),
    ("lgb_lc64.cu", ["--fmad=false"]),
    ("lgb_lb2.cu", ["--fmad=false"]),
    ("lgb_sk.cu", []),
    ("lgb_lc32.cu", []),
    ("lgb_fused32.cu", []),
    ("lgb_cnn.cu", []),
    ("lgb_coarse.cu", []),
]
C_SOURCES = ["ludwig_gb.c", "ludwig_gb_cnn.c", "ludwig_gb_io.c"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _run(cmd):
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd),
                                                         out.stdout,
                                                         out.stderr))
    return out.stdout + out.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Compile every CUDA and C source and link libludwig_gb.so."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
               if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "ludwig_gb.h"))

    jobs = []
    objs = []
    for src, flags in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, "-std=c++17", "-O3", "-lineinfo"] + ARCH +
                        flags + ["-Xcompiler", "-fPIC", "-I", CSRC,
                                 "-I", INCLUDE, "-c", s, "-o", o])
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".c", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["gcc", "-std=gnu11", "-O2", "-fPIC", "-Wall",
                         "-ffp-contract=off", "-I", CSRC, "-I", INCLUDE,
                         "-I", os.path.join(cuda, "include"), "-c", s,
                         "-o", o])
    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as ex:
        for log in ex.map(_run, jobs):
            if verbose and log.strip():
                print(log)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, "-shared"] + ARCH + objs +
             ["-o", LIB, "-lcudart"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
    print(LIB)
