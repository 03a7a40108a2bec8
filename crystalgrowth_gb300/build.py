"""Build libkobayashi_gpu.so in-tree with nvcc for sm_103a.

Every ``csrc/*.cu`` file is compiled in parallel to ``_build/*.o`` and linked
into ``crystalgrowth_gb300/libkobayashi_gpu.so``.  Device code is compiled with
``-fmad=false`` and host code with ``-ffp-contract=off`` so that no a*b+c is
fused behind the source's back: the kernels must reproduce the CPU oracle's
IEEE FP64 results bit for bit.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libkobayashi_gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libkobayashi_gpu.so")
    return cand


def cflags():
    extra = os.environ.get("KG_NVCC_EXTRA", "").split()
    return ARCH + extra + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _deps():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.h")) +
                  glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(ROOT, "include", "*.h")) +
                  [os.path.abspath(__file__)])


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + cflags() + (["-Xptxas", "-v"] if verbose_ptxas else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (os.path.basename(src), r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose_ptxas=False, quiet=True):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        res = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    logs = "".join(r[1] for r in res)
    if verbose_ptxas:
        with open(os.path.join(BUILD, "ptxas.log"), "w") as f:
            f.write(logs)
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [r[0] for r in res] + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    if not quiet:
        print(LIB)
    return LIB


# Compile-time switches of the kernels and the setting each one ships with.  Every other setting
# computes the same bits (they exist for A/B measurements; the defaults are the measured winners).
SWITCHES = {"KG_BITS_ASM": 1, "KG_GDIV": 1, "KG_FAR": 1, "KG_FUSE": 1, "KG_QUIET": 3, "KG_ABSORB": 1,
            "KG_IDIV_SUBN": 1, "KG_SLOW_NOINLINE": 1, "KG_TMA": 1}
# the plain build: every shortcut and every switch in its other setting
PLAIN = {"KG_BITS_ASM": 0, "KG_GDIV": 0, "KG_FAR": 0, "KG_FUSE": 0, "KG_QUIET": 0, "KG_ABSORB": 0,
         "KG_IDIV_SUBN": 0, "KG_SLOW_NOINLINE": 0, "KG_TMA": 0}


def build_variant(lib_path, defines):
    """Build the library with extra -D definitions into lib_path (object files beside it)."""
    bdir = os.path.join(os.path.dirname(os.path.abspath(lib_path)), "_obj")
    os.makedirs(bdir, exist_ok=True)
    flags = ["-D%s=%s" % kv for kv in sorted(defines.items())]
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))

    def one(src):
        obj = os.path.join(bdir, os.path.basename(src)[:-3] + ".o")
        r = subprocess.run([nvcc()] + cflags() + flags + ["-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s with %s:\n%s" % (os.path.basename(src), flags, r.stderr))
        return obj
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(one, srcs))
    r = subprocess.run([nvcc()] + ARCH + ["-shared", "-o", lib_path] + objs + ["-lcudart"], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    return lib_path


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, quiet=False)
    if "-v" in sys.argv:
        print(open(os.path.join(BUILD, "ptxas.log")).read())
