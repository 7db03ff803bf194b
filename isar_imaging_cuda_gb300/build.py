"""In-tree build of libisar_gb300.so for sm_103a (nvcc, no CMake).

Translation units are compiled in parallel into isar_imaging_cuda_gb300/_lib
and linked against the shared CUDA runtime.  Rebuilds only when a source or
header is newer than the library.
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
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libisar_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for p in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _deps():
    return sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h")) + [os.path.abspath(__file__)]


def _compile(nvcc, src, obj, verbose):
    cmd = [nvcc] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
                           "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc, "-x", "cu"] + cmd[1:]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-8000:]))
    return r.stderr


def build(force=False, verbose=False):
    """Compiles every CUDA translation unit for sm_103a and links the library."""
    os.makedirs(LIBDIR, exist_ok=True)
    if not force and os.path.exists(LIB):
        if os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in _deps()):
            return LIB
    nvcc = _nvcc()
    srcs = sources()
    objs = [os.path.join(LIBDIR, os.path.basename(s) + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        logs = list(ex.map(lambda so: _compile(nvcc, so[0], so[1], verbose), zip(srcs, objs)))
    if verbose:
        for s, lg in zip(srcs, logs):
            sys.stderr.write("== %s\n%s" % (os.path.basename(s), lg))
    home = _cuda_home(nvcc)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs + \
        ["-Xlinker", "-rpath," + os.path.join(home, "lib64"), "-Xlinker", "-rpath," + os.path.join(home, "lib")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr[-4000:]))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
