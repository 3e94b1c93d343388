"""Build libvfps.so (CUDA kernels + C ABI) for sm_103a, in-tree.

Each .cu under inovesa_gb300/csrc is compiled to an object in parallel and
linked into inovesa_gb300/_build/libvfps.so.  Only nvcc and the CUDA
runtime are needed; PyTorch is not involved.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libvfps.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(ROOT, "include", "vfps.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    """Compile every CUDA translation unit and link libvfps.so."""
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    # host code rounds like the reference's CPU build on x86-64 and aarch64:
    # no contraction of float multiply-adds into FMA
    common = ARCH + ["-lineinfo", "-O3", "-std=c++17",
                     "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
                     "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    common += list(extra_flags)

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        cmd = [cc] + common + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s"
                               % (src, r.stdout, r.stderr))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


DRIVER = os.path.join(OUT, "vfps_solver")


def build_driver(force=False):
    """The C++ solver driver over include/vfps.hpp, linked to libvfps.so
    (found next to it at run time)."""
    lib = build()
    src = os.path.join(HERE, "cpp", "vfps_solver.cpp")
    deps = [src, lib, os.path.join(ROOT, "include", "vfps.hpp"),
            os.path.join(ROOT, "include", "vfps.h")]
    if not force and not _stale(DRIVER, deps):
        return DRIVER
    cxx = shutil.which("g++") or "g++"
    tmp = DRIVER + ".tmp%d" % os.getpid()
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-Wextra", "-I",
           os.path.join(ROOT, "include"), src, "-L", OUT, "-lvfps",
           "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, DRIVER)
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra_flags=[a for a in sys.argv[1:] if a.startswith("-X")]))
