"""CPU build of the reference's own sources (TEST INFRASTRUCTURE ONLY).

Recipe: every translation unit of Junf137/isar_imaging_cuda/isar_imaging
(common.cu, high_speed_compensation.cu, range_alignment.cu,
phase_adjustment.cu, mtrc.cu, isar_main.cu, isar_imaging_export.cpp) is read
where it lies under the reference checkout, its `kernel<<<cfg>>>(args)`
launches are rewritten to `EMU_LAUNCH(kernel, cfg)(args)` on the way into the
compiler (piped through stdin; no copy of the sources is written anywhere),
and it is compiled by g++ as C++20 against the real CUDA headers plus the
emulation headers in include/: kernels run as host loops (fibers where they
use __syncthreads), Thrust runs on its CPP backend, cuFFT and cuBLAS calls go
to double-precision host stand-ins with the same conventions.  Outputs go to
oracle/_ref/libisar_ref_emu.so (x86_64, this container only).

The build needs no GPU.  It is used to generate the golden vectors under
tests/golden/ that pin the FP64 restatement (isar_oracle.c) to the
reference's own control flow, kernels and reductions.
"""
import concurrent.futures as cf
import ctypes as C
import os
import re
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libisar_ref_emu.so")
# The reference checkout's isar_imaging directory comes from the environment
# only (ISAR_REFERENCE_DIR); the recipes that build this emulation set it.


def ref_dir():
    return os.environ.get("ISAR_REFERENCE_DIR", "")
REF_SOURCES = ["common.cu", "high_speed_compensation.cu", "range_alignment.cu", "phase_adjustment.cu",
               "mtrc.cu", "isar_main.cu", "isar_imaging_export.cpp"]
_LAUNCH = re.compile(r"([A-Za-z_]\w*)\s*<<\s*<(.*)>>\s*>\s*\(")


def reference_present():
    d = ref_dir()
    return bool(d) and all(os.path.exists(os.path.join(d, s)) for s in REF_SOURCES)


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    home = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    inc = os.path.join(home, "include")
    cccl = [os.path.join(home, "include", "cccl")]
    cccl += [os.path.join(home, "targets", d, "include", "cccl") for d in ("x86_64-linux", "sbsa-linux")]
    return [inc] + [d for d in cccl if os.path.isdir(d)]


def _flags():
    f = ["-std=c++20", "-O2", "-fPIC", "-w", "-ffp-contract=off", "-fno-fast-math",
         "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP",
         "-D__global__=", "-D__device__=", "-D__host__=", "-D__shared__=", "-D__STORAGE__=extern",
         "-D__declspec(x)=",
         "-include", os.path.join(HERE, "include", "emu_pre.h"),
         "-I", os.path.join(HERE, "include"), "-I", ref_dir()]
    for d in _cuda_include():
        f += ["-I", d]
    return f


def transform(text):
    """Rewrites CUDA launch syntax into the emulation's launcher call."""
    return "\n".join(_LAUNCH.sub(r"EMU_LAUNCH(\1, \2)(", ln) for ln in text.split("\n"))


def _compile_ref(src):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    text = transform(open(os.path.join(ref_dir(), src), encoding="utf-8-sig").read())
    cmd = ["g++"] + _flags() + ["-x", "c++", "-", "-c", "-o", obj]
    r = subprocess.run(cmd, input=text, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compiling %s failed:\n%s" % (src, r.stderr[-6000:]))
    return obj


def _compile_own(src):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    cmd = ["g++"] + _flags() + ["-c", os.path.join(HERE, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compiling %s failed:\n%s" % (src, r.stderr[-6000:]))
    return obj


def build(force=False):
    """Builds oracle/_ref/libisar_ref_emu.so from the reference sources."""
    if not reference_present():
        raise RuntimeError("reference sources not found (ISAR_REFERENCE_DIR=%r)" % ref_dir())
    if not force and os.path.exists(LIB):
        mine = [os.path.join(HERE, p) for p in ("emu_runtime.cpp", "ref_driver.cpp", "__init__.py")]
        mine += [os.path.join(HERE, "include", p) for p in os.listdir(os.path.join(HERE, "include"))]
        if os.path.getmtime(LIB) >= max(os.path.getmtime(p) for p in mine):
            return LIB
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(_compile_ref, REF_SOURCES))
        objs += list(ex.map(_compile_own, ["emu_runtime.cpp", "ref_driver.cpp"]))
    tmp = LIB + ".tmp%d" % os.getpid()
    r = subprocess.run(["g++", "-shared", "-Wl,--no-undefined", "-o", tmp] + objs + ["-lm", "-lpthread"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("linking the emulated reference failed:\n%s" % r.stderr[-6000:])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _lib.ref_frame.restype = C.c_int
        _lib.ref_frame.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_longlong, C.c_longlong,
                                   C.c_double, C.c_longlong, C.c_int, C.c_int, C.c_int,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.ref_hrrp.restype = C.c_int
        _lib.ref_hrrp.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p]
        _lib.ref_parse.restype = C.c_int
        _lib.ref_parse.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_char_p]
        _lib.ref_extract.restype = C.c_int
        _lib.ref_extract.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_char_p]
        _lib.ref_pulse_compress.restype = C.c_int
        _lib.ref_pulse_compress.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_longlong, C.c_longlong,
                                            C.c_double, C.c_longlong, C.c_void_p]
    return _lib


def frame(echo, velocity, M, N, B=1.0e9, fc=10.0e9, Fs=100.0e6, Tp=None, hpc=False, mtrc=False,
          checkpoints=True):
    """Runs the reference on one frame.  Returns dict(img, ra, cut, fe)."""
    if Tp is None:
        Tp = N / Fs
    e = np.ascontiguousarray(echo, np.complex64)
    v = np.ascontiguousarray(velocity if velocity is not None else np.zeros(M), np.float64)
    img = np.zeros((M, 512), np.float32)
    ra = np.zeros((M, N), np.complex64) if checkpoints else None
    cut = np.zeros((M, 512), np.complex64) if checkpoints else None
    fe = np.zeros((M, 512), np.complex64) if checkpoints else None
    p = lambda a: None if a is None else a.ctypes.data
    rc = lib().ref_frame(p(e), p(v), M, N, int(B), int(fc), float(Tp), int(Fs), 2, int(hpc), int(mtrc),
                         p(img), p(ra), p(cut), p(fe))
    if rc != 0:
        raise RuntimeError("reference rejected the frame (rc=%d)" % rc)
    return dict(img=img, ra=ra, cut=cut, fe=fe)


def pulse_compress(ad, velocity, B, fc, Tp, Fs):
    """IFDS pulse compression of each pulse by the reference's pulseCompression
    class.  ad: int16 [P, 2*iq_len] (I, Q interleaved).  Returns complex64
    [P, 4096]."""
    ad = np.ascontiguousarray(ad, np.int16)
    P, two_l = ad.shape
    out = np.zeros((P, 4096), np.complex64)
    for p in range(P):
        iq = np.ascontiguousarray(ad[p].astype(np.float32))
        o = np.zeros(4096, np.complex64)
        rc = lib().ref_pulse_compress(iq.ctypes.data, two_l // 2, float(velocity[p]), int(B), int(fc), float(Tp),
                                      int(Fs), o.ctypes.data)
        if rc != 0:
            raise RuntimeError("reference pulse compression failed (rc=%d)" % rc)
        out[p] = o
    return out


def read_dump(path, dtypes):
    """Count-prefixed arrays written by the drivers' dump(): per array an
    int64 element count, then the elements (dtypes in order)."""
    out = []
    with open(path, "rb") as f:
        for dt in dtypes:
            n = int(np.frombuffer(f.read(8), np.int64)[0])
            out.append(np.frombuffer(f.read(n * np.dtype(dt).itemsize), dt).copy())
    return out


def parse(directory, polar_type=1, data_type=2):
    """dataParsing by the reference on the .wbd files in `directory`: returns
    (frame_len, frame_num, dataN float64, turnAngle float32)."""
    out = os.path.join(OUT, "parse_%d.bin" % os.getpid())
    rc = lib().ref_parse(directory.encode(), polar_type, data_type, out.encode())
    if rc != 0:
        raise RuntimeError("reference dataParsing failed (rc=%d)" % rc)
    fl, dn, ta = read_dump(out, (np.int32, np.float64, np.float32))
    os.remove(out)
    return int(fl[0]), int(fl[1]), dn, ta


def extract(directory, window_len, window_head, sampling_stride=1, polar_type=1, data_type=2):
    """dataParsing + imagingMemInit + one dataExtracting by the reference:
    returns (dataWFileSn int32, dataNOut float64, turnAngleOut float32,
    dataW complex64)."""
    out = os.path.join(OUT, "extract_%d.bin" % os.getpid())
    rc = lib().ref_extract(directory.encode(), polar_type, data_type, window_len, window_head, sampling_stride,
                           out.encode())
    if rc != 0:
        raise RuntimeError("reference dataExtracting failed (rc=%d)" % rc)
    sn, dn, ta, dw = read_dump(out, (np.int32, np.float64, np.float32, np.float32))
    os.remove(out)
    return sn, dn, ta, dw.view(np.complex64)


def hrrp(echo, data_type=2):
    """getHRRP of a complex64 [M, N] frame by the reference (complex64 out)."""
    e = np.ascontiguousarray(echo, np.complex64)
    M, N = e.shape
    out = np.zeros((M, N), np.complex64)
    rc = lib().ref_hrrp(e.ctypes.data, M, N, int(data_type), out.ctypes.data)
    if rc != 0:
        raise RuntimeError("reference getHRRP failed (rc=%d)" % rc)
    return out
